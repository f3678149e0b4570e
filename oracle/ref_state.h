// ORACLE -- test infrastructure only.  A CPU (FP64, sequential) restatement of
// the cg-gcmc-bd hot-path routines of the BROMOC reference, used by tests/,
// __graft_entry__.smoke() and the CPU-baseline leg of bench.py as the
// reference the GPU results are compared with.
// Nothing in the product links or calls this code.
//
// Parity status: the reference (Fortran 90) cannot be compiled with the
// toolchains at hand (C, C++ and CUDA only), and it ships no golden
// vectors.  This restatement is pinned only by the reference's own built-in
// known-answer procedures -- TEST (central finite-difference forces,
// testfirst.f90:35-85) and ENERGY == 1/2 sum INTERACT
// (shell_simul.f90:2688-2696) -- so its parity with the reference's outputs
// is "parity unpinned".
//
// State mirrors the Fortran modules (grandmod, gsbpmod, efpmod, extramod,
// nucleotmod); particle arrays are 1-based like the Fortran.
#pragma once
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include "../include/bromoc_gpu.h"

namespace bref {

constexpr double pi = 3.14159265358979323846264338327950288419716939937510;
constexpr double twopi = 2.0 * pi;
// constamod.f90:73-84
constexpr double kboltz = 1.380648813E-23;
constexpr double angstrom = 1E-10;
constexpr double avogadro = 6.0221412927E23;
constexpr double kcal = 4184.0;
constexpr double kcalmol = kcal / avogadro;
constexpr double Coulomb = 1.60217656535E-19;
constexpr double epermit = 8.854187817620E-12;
inline double celec_value() {
  return Coulomb * Coulomb / (4.0 * pi * epermit * kcalmol * angstrom);
}
constexpr double rsmall = 1E-3;

// Fortran x**3 and x**6 for default-real x
inline double pow3(double v) { return v * v * v; }
inline double pow6(double v) {
  double v2 = v * v;
  return v2 * v2 * v2;
}

struct Grid {
  int nclx = 0, ncly = 0, nclz = 0;
  double dcel = 0, idcel = 0, tranx = 0, trany = 0, tranz = 0;
  double xbcen = 0, ybcen = 0, zbcen = 0;
  void set(const bromoc_grid &g);
};

// DNA bonded and Go-like term lists (nucleotmod.f90), 1-based sites; a
// term's sites are consecutive in its list
struct Nucl {
  bool on = false;
  double epsnuc = 0, scalepairing = 1, fctn = 0, kappa = 0, ikappa = 0, epsolv = 0;
  int qdeby = 0;
  bool qsolv = false, qunsplit = false;
  int nsites1st = 0;
  std::vector<int> bond, angle, dihe, stack, bp, ex, qq, slv;
  std::vector<double> distbond, valangle, valdihe, sgstack, sgbp, sgex;
  std::vector<uint8_t> bpgc;
  std::vector<int> sn, csn;
  std::vector<double> af, kx, ky, kz, contrx, contry, contrz;
  int qnotr[3] = {0, 0, 0};  // NOTRAN axes and centres
  double notr[3] = {0, 0, 0};
};

// Reaction field of the MMIJ basis (gsbpmod): RECTBOX Legendre products or
// SPHERE multipoles; basis vectors 0-based, mmij row-major ntpol x ntpol
struct Mmij {
  bool on = false, rect = true;
  int xnpol = 0, ynpol = 0, znpol = 0, nmpol = 0, ntpol = 0;
  std::vector<int> lstpx, lstpy, lstpz, lstpl, lstpm;
  std::vector<double> bnorm, mmij;
  double xscal = 0, yscal = 0, zscal = 0, xmin = 0, xmax = 0, ymin = 0, ymax = 0, zmin = 0,
         zmax = 0, rfscal = 1, srdist = 0;
};
void mmij_basis(Mmij &m);

struct State {
  std::string err;
  double celec = celec_value();
  int capacity = 23000;
  // SYSTEM
  bromoc_system sys{};
  bool have_sys = false;
  double ikbt = 0, kbtdt = 0;
  double lx2m = 0, lx2p = 0, ly2m = 0, ly2p = 0, lz2m = 0, lz2p = 0;
  double rsphe2 = 0, iecx = 0, iecy = 0;
  // extension mode (no counterpart in the reference): minimum-image periodic
  // box and a plain cutoff on ion pairs, positions wrapped after each move
  bool periodic = false;
  double rcut2 = 0;
  // types (1-based)
  int ntype = 0, nold = 0, nttyp = 0, ndna = 0, nion = 0, ndnaxnion = 0;
  std::vector<int> nwtype;
  std::vector<double> cg, diffusion, fact1a, fact2a;
  bool have_types = false;
  // pair laws (1-based by is)
  int ntc = 0;
  std::vector<uint8_t> qchr, qlj, qsrpmfi, qefpot;
  std::vector<double> fct, epp4, sgp2, c0, c1, c2, c3, c4;
  double rth = 0, srpx = 0, srpk = 0, srpy = 0;
  int cnt = 0;
  std::vector<double> ep;  // ep(1:3, 1:cnt) -> ep[3*(k-1) + (m-1)]
  std::vector<double> sc, dm2, dmi;
  std::vector<int> nxi;
  double res = 0, ires = 0;
  bool have_pairs = false;
  // sites
  int nsites = 0;
  std::vector<int> typtyp, site_phiv_map;
  std::vector<double> sitecharge;
  std::vector<uint8_t> stfree;
  // particles (1-based)
  int ntot = 0, nfix = 0;
  std::vector<double> x, y, z, fx, fy, fz;
  std::vector<int> typei, ibuffer;
  std::vector<double> dids;  // dids(1:5, i) -> dids[5*(i-1) + (m-1)]
  // static field
  bool qphix = false;
  Grid g1;
  std::vector<float> phix;
  // repulsion
  bool qphiv = false, qtrln = true, qnmcden = false, qsvdw = false;
  Grid g2;
  std::vector<int8_t> phiv;
  int phiv_nmaps = 1;
  double svdw = 0, vzmin = 0, vzmax = 0, thold8 = 8, thold27 = 27;
  std::vector<int> phiv_map_of_type;  // 1-based by ion type
  std::vector<double> scal;           // 1-based by combined type
  // RFPAR
  bool qrfpar = false, qrfpsin = true;
  Grid g3;
  std::vector<float> gsrfen, greff;
  double sqrfac = 0;
  std::vector<int> rfpar_map_of_type;  // 1-based by ion type
  // membrane
  bool qmemb = false, qpore = false;
  double voltage = 0, afact = 0, ikappa = 0, ceps = 0, zmemb1 = 0, zmemb2 = 0;
  std::vector<double> ampl1, p1a, p1b, ampl2, p2a, p2b, rcylinder;
  // diffusion models
  bromoc_diffusion dif{};
  std::vector<double> ampl3, p3, xs, ys, sb, scc, sd;
  bool have_dif = false;
  // countions
  int cntpts = 0;
  std::vector<double> zcont;
  std::vector<int> nforward, nbackward;  // [(itype-nold-1)*cntpts + (j-1)]
  // GCMC buffers (1-based by ib)
  int nbuffer = 0;
  std::vector<int> ibfftyp, nat, ntotat, ninsert, nremove;
  std::vector<double> avnum, mu, kb, lzmin, lzmax, rmin, rmax;
  std::vector<uint8_t> qbufferbias;
  std::vector<int> prob;  // prob(ib, 0:capacity) -> [(ib-1)*(capacity+1) + n]
  // energies (grandmod / gsbpmod)
  double ener = 0, eelec = 0, evdw = 0, esrpmf = 0, esrpmfmx = 0, eefpot = 0,
         eefpotmx = 0, ememb = 0, egsbpa = 0, egsbpb = 0, evdwgd = 0,
         erfpar = 0, eqqmx = 0, evdwmx = 0;
  std::vector<int> warn;  // 1-based by combined type
  // DNA bonded / Go-like terms (nucleotmod)
  Nucl nuc;
  // MMIJ reaction field (gsbpmod)
  Mmij mm;
  double ebond = 0, eang = 0, edihe = 0, estack = 0, ebp = 0, eex = 0, eqq = 0,
         esolv = 0, econ = 0;

  bool qpar() const { return have_types && ntype > nold; }  // PARTICLES given
  // extension mode: nearest periodic image of a separation
  void min_image(double &dx, double &dy, double &dz) const {
    if (!periodic) return;
    dx -= sys.lx * std::rint(dx / sys.lx);
    dy -= sys.ly * std::rint(dy / sys.ly);
    dz -= sys.lz * std::rint(dz / sys.lz);
  }
  bool qnucl() const { return nsites > 0; }
  void resize_particles(int cap);
};

// nindex.f90:19-35
int nindex(const State &s, int itype, int jtype);
// polynom.f90:172-254
void gety(const State &s, int is, double x2, double &y, double &x);
void getyd(const State &s, int is, double x2, double &y, double &yp,
           double &x);
// polynom.f90:20-169
void squarespline(int n, const double *x, const double *y, double *p,
                  double d1, double d2, double dd2);
// splinepot.f90:19-96 (one pair; p is the pair's slice of ep)
void splinepot(int nn, const double *xx, const double *yy, double fct,
               bool qchr, double *p, double *sc3, double *dm2o, double *dmio);

void energy(State &s, uint32_t mask, bool qforces);
// grandmod.f90:74-98
bool outbox(const State &s, double xi, double yi, double zi);
// energy.mono.f90:196-582 and interact.f90:211-334 (ref_nucl.cpp)
void nucl_energy(State &s, uint32_t mask, bool qforces);
void nucl_interact(const State &s, uint32_t mask, int j, double &dener);
// rect_rf1/sphe_rf1 (egsbpb, forces) and rect_rf0/sphe_rf0 (ref_mmij.cpp)
void mmij_energy(State &s, bool qforces);
double mmij_interact(const State &s, double xj, double yj, double zj, int j, int jtype);
void membrane(State &s, bool qforces);
void staticf1(State &s, bool qforces);
void vdwgd1trln(State &s, bool qforces);
void vdwgd1spln(State &s, bool qforces);
void rfparion(State &s, bool qforces);
void staticf0(State &s, double xj, double yj, double zj, int j, int jtype);
void vdwgd0trln(State &s, double xj, double yj, double zj, int j, int jtype,
                int jtype2, bool qalert);
void vdwgd0spln(State &s, double xj, double yj, double zj, int j, int jtype,
                int jtype2, bool qalert);
void rfparionj(State &s, double xj, double yj, double zj, int j, int jtype);
void interact(State &s, uint32_t mask, double &dener, double xj, double yj,
              double zj, int jtype, int j, bool qalert);
void switch1(double &sw, double &dsw, double z, double p1, double ip1,
             double zmemb1, double zmemb2);
void switch2(double &sw, double &dsw, double r2, double radius, double p2,
             double ip2, double &r);
void fixcoor(const State &s, double &xi, double &yi, double &zi);
void dynamics(State &s, int variant, uint64_t seed, uint64_t step);
void grand(State &s, uint32_t mask, int ngcmc, uint64_t seed, uint64_t icycle,
           double &dener_sum);
// count.f90:19-95 (false: a particle lies outside the system)
bool count(State &s);

// noise: Philox4x32-10 (Salmon et al., SC'11) + Box-Muller cos branch
void philox4x32_10(const uint32_t ctr[4], const uint32_t key[2],
                   uint32_t out[4]);
double bd_gauss(uint64_t seed, uint64_t step, uint32_t slot, int comp);
double gcmc_uniform(uint64_t seed, uint64_t cycle, uint32_t attempt,
                    uint32_t draw);
double mc_uniform(uint64_t seed, uint64_t cycle, uint32_t move, uint32_t draw);
// metropolis.f90:31-55 with move.f90:19-45; at most kMcTries draws of a
// position inside the system per move (the reference draws until one is)
constexpr int kMcTries = 1000;
void metropolis(State &s, uint32_t mask, int nmcm, double mcmax, uint64_t seed,
                uint64_t cycle, double &dener_sum, int &naccept);

}  // namespace bref
