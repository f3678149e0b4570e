// Kernel parameter block: every kernel receives one KP by value.  Device
// pointers only; the host-side context (api.cu) owns the allocations.
#pragma once
#include "common.cuh"

namespace bgpu {

// Relative window around the SRPMF boundaries on r^2 within which the FP32
// pair path takes its branch from the pair's FP64 r^2 (srp_branch).
constexpr double kSrpWin = 4e-6;

struct Grid3 {
  int nclx, ncly, nclz;
  double dcel, idcel, tranx, trany, tranz, xbcen, ybcen, zbcen;
};

struct PairParamF {  // FP32 copy of PairParam for the single-precision path
  float fct, epp4, sgp2, c0, c1, c2, c3, c4, sc0, sc1, sc2, dm2lo, dm2hi, dmi;
  int flags, nxi;
};

// One coordinate axis of one grid for the float-float cell search (ff.cuh).
struct AxisF {
  float oh, ol;    // tran - bcen as hi + lo
  float dh, dl;    // dcel as hi + lo
  float idc;       // 1 / dcel
  float ubh, ubl;  // in-map test: lb <= position <= ub, each as hi + lo
  float lbh, lbl;
  int ncl;
};

// System shape for fixcoor in float-float (fixcoor.f90).
struct BoxF {
  int shape;           // 0 box, 1 sphere, 2 elliptic cylinder
  float rsphe, rsphe2, iecx, iecy;
  float bh[6], bl[6];  // box bounds x-,x+,y-,y+,z-,z+ (hi, lo)
  float ch[3], cl[3];  // shape centre (hi, lo)
  int periodic;        // extension mode: wrap instead of clamp (box only)
  float Lh[3], Ll[3];  // box lengths (hi, lo)
};

// Single-precision constants of the FP32 path, filled on the host so that
// no kernel of that path converts a double.
struct F32C {
  // lanes 3m+a: axis a of grid m (0 static field, 1 repulsion, 2 RFPAR);
  // 9..11: the repulsion grid for the B-spline stencil
  AxisF ax[12];
  float celec, sqrfac, thold8, thold27, kbtdt, bdmax, fact0n1, fact0n2;
  BoxF box;
  float L[3], iL[3], rc2;  // extension mode: box lengths, their inverses, cutoff^2
};

// Float-float twins (value = x + y) of what GRAND's ΔE reads, filled on the
// host so that the GRAND kernel converts no constant.
struct PairFF {  // PairParam; c3pi = c3 * pi as the FP64 law forms it
  float2 fct, epp4, sgp2, c0, c1, c2, c3pi, c4, sc0, sc1, sc2, dm2lo, dm2hi, dmi;
  int flags, nxi, npieces, pad;
};
struct GridFF {  // Grid3: in-map bounds bcen -+ tran, offsets tran - bcen, cell size
  float2 ub[3], lb[3], o[3];
  float2 dcel, idcel;
  int ncl[3];
};
struct FFC {
  GridFF g[3];    // static field, repulsion, RFPAR
  float2 sqrfac, thold8, thold27, vzmin, vzmax;
  float2 rth, srpx, srpk, srpy, ires, ikbt;
  float2 L[3];    // extension mode: box lengths
  float iL[3];    //   their inverses (nearest float)
  float2 rc2;     //   cutoff on r^2
};
// A GRAND trial as its pair terms read it, in float-float.
struct TrialFF {
  float2 x, y, z;
  float2 a;       // celec q_trial srfe reff: factor of the RFPAR cross term
  float2 b;       // reff^2 of the trial
  int valid, j, jt2, rf;  // rf: the cross term is on
};
static_assert(sizeof(TrialFF) % 8 == 0 && alignof(TrialFF) == 8, "TrialFF is read as uint2");

// DNA bonded and Go-like terms between sites (nucleotmod.f90), as one term
// list in kind order: bond, angle, torsion, stack, base pair, excluded
// volume, P-P electrostatics, solvent, applied force (APFOR).
constexpr int kNucKinds = 9;
struct NucDev {
  int nterm;                    // 0: none
  int off[kNucKinds + 1];       // first term of each kind
  const int4 *site;             // [nterm] 0-based sites (-1 unused); base pair: .z = G-C
  const double *par;            // [nterm] d0, theta0, phi0 or sigma
  const double *af;             // [3*afn] applied forces
  double *te;                   // [nterm] term energies
  double *tf;                   // [nterm*4*3] force of term t on its site m at (4t+m)*3
  const int *csr_start;         // [nsites+1] each site's entries in csr_ent
  const int *csr_ent;           // entries 4t+m in ascending t
  double epsnuc, scalepairing, fctn, kappa, ikappa, epsolv;
  int qdeby, qsolv;
  int ctn, qunsplit, nsites1st;
  const int *csn;               // [ctn] CONTRANS site (1-based) or 0 for the centre
  const double *ck;             // [3*ctn] (kx, ky, kz) per entry
  const double *cc;             // [3*(ctn+1)] anchors (x, y, z) per entry
  double *cf;                   // [8] centre force per strand and axis, econ
  int qnotr[3];                 // NOTRAN: recentre the sites along these axes
  double notr[3];
};

// Reaction field of the MMIJ basis (gsbpmod): RECTBOX Legendre products or
// SPHERE multipoles, FP64; per-particle basis tables (row cap: INTERACT's
// trial), the coefficient vector and M coef.
struct MmijDev {
  int on, rect;
  int nx, ny, nz, nmpol, ntpol;  // RECTBOX orders per axis; SPHERE nmpol
  int tabw;                      // doubles per table row
  const int3 *lst;               // [ntpol] (lx, ly, lz) or (l, m, 0)
  const double *bnorm;           // [ntpol]
  const double *m;               // [ntpol*ntpol] symmetric
  double xscal, yscal, zscal, xmax, ymax, zmax, rfscal, srdist2;
  double *tab;                   // [(cap+1)*tabw]
  unsigned char *in;             // [cap+1] in the region
  double *ist;                   // [cap+2] SPHERE 10/sin(theta); [cap+1]: the last ion's
  double *coefp;                 // [nchunk*ntpol] per-chunk partial sums
  double *coef, *coef2, *mq, *rowe;  // [ntpol]
};

struct KP {
  // ---- sizes (host-known) ----
  int cap, nsites, nfix, ntype, nold, nttyp, ndna, ntc;
  DevState *st;   // live ntot, buffer counters, error flags
  // ---- system ----
  int shape, qcountion;
  // extension mode (no counterpart in the reference): minimum-image periodic
  // box and a plain cutoff rc2 (on r^2) for ion pairs; moves wrap
  int periodic;
  double rc2;
  double lx, ly, lz, cx, cy, cz, rsphe, rsphe2, iecx, iecy;
  double lx2m, lx2p, ly2m, ly2p, lz2m, lz2p;
  double kbtdt, ikbt, dt, bdmax;
  double celec;
  // ---- particles ----
  double *x, *y, *z;
  int *typei, *ibuffer;
  double *fx, *fy, *fz;   // assembled forces [cap]
  // ---- types (1-based arrays by ion type / combined type) ----
  const int *nwtype;      // [ntype+1]
  const double *cg, *diffusion, *fact1a, *fact2a;  // [ntype+1]
  // ---- pair laws ----
  const PairParam *pp;    // [ntc]
  const PairParamF *ppf;  // [ntc]
  // [4*ntc] packed FP32 laws: (fct, epp4, sgp2, flags|npieces<<8),
  // (c0, c1, c2, c3), (c4, sc0, sc1, sc2), (dm2lo, dm2hi, dmi, nxi)
  const float4 *ppk;
  const int *pidx;        // [nttyp*nttyp] 0-based pair index, -1 none
  // dense ion-ion law table for the FP32 pair kernel: [nion_t * nion_t] of
  // (fct, 6 epp4, sgp2, rth or -1), fct/epp4 zeroed where the pair has no
  // Coulomb/LJ term, rth (the SRPMF cutoff on r^2, widened by srp_branch's
  // FP64 decision window) where it has SRPMF;
  // ipq_ok when it applies (no tabulated ion-ion law, nion_t <= kIonTabTypes)
  const float4 *ipq;
  int nion_t, ipq_ok;
  const double *ep;       // [3*cnt] reference form (p1,p2,p3)
  const float4 *ep32;     // [cnt] local form (a, b, c, x_k)
  int cnt;
  double rth, srpx, srpk, srpy, res, ires;
  float rthf, srpxf, srpkf, srpyf, iresf;  // FP32 copies for the fast path
  // the SRPMF boundaries on r^2 (taper start srpx^2, cutoff rth) with the
  // window around each in which srp_branch decides in FP64: below, above
  float srpx2lo, srpx2hi, rthlo, rthhi;
  // ---- sites ----
  const int *typtyp;      // [nsites] 1-based combined type
  const double *sitecharge;
  const uint8_t *stfree;
  const int *site_map;    // [nsites] nmcden map or nullptr
  NucDev nuc;
  MmijDev mm;
  // ---- static field ----
  int qphix;
  Grid3 g1;
  const float *phix;
  // ---- repulsion ----
  int qphiv, qtrln, qnmcden, qsvdw;
  Grid3 g2;
  const int8_t *phiv;
  double svdw, vzmin, vzmax, thold8, thold27;
  const int *phiv_map_of_type;  // [ntype+1]
  const double *scal;           // [nttyp+1]
  // ---- RFPAR ----
  int qrfpar, qrfpsin;
  Grid3 g3;
  const float *gsrfen, *greff;
  double sqrfac;
  const int *rfpar_map_of_type; // [ntype+1]
  double *rf_srfe, *rf_reff;    // [cap] per-particle gathers
  double *rf_d1, *rf_d2;        // [3*cap] derivatives
  uint8_t *rf_in;               // [cap] in-grid flag
  // ---- membrane ----
  int qmemb, qpore;
  double voltage, afact, ikappa, ceps, zmemb1, zmemb2;
  const double *ampl1, *p1a, *p1b, *ampl2, *p2a, *p2b, *rcyl;  // [nttyp+1]
  // ---- diffusion models ----
  double plength2, pcenter;
  const double *ampl3, *p3;     // [ntype+1]
  int nspline;
  const double *xs, *ys, *sb, *scc, *sd;  // [nspline+1] 1-based
  double diff0, ibeta, diffcutoff, fact0n1, fact0n2;
  int qdnafree, qproxdiff;
  double *dids;                 // [5*cap]
  // ---- countions ----
  int cntpts;
  const double *zcont;          // [cntpts]
  int *nforward, *nbackward;    // [(ntype-nold)*cntpts]
  // ---- GCMC ----
  int nbuffer;
  const int *ibfftyp;           // [nbuffer+1]
  const double *avnum, *mu, *kbb, *lzmin, *lzmax, *rmin, *rmax;
  const uint8_t *qbufferbias;
  int *prob;                    // [nbuffer*(cap+1)]
  Trial *trial;                 // [kSpec] INTERACT's trial; GRAND's round trials
  GrandRound *ground;           // GRAND's round header
  double2 *gc_rf;               // [cap] RFPAR (srfe, reff) of each ion for
                                // INTERACT's cross term, (0,0) off the map
  // ---- scratch ----
  double *ffield;               // [3*cap] single-particle field forces
  double *fii;                  // [nchunk_ii*3*cap] ion-ion partial forces
  int nchunk_ii, chunk_ii;
  double *fis;                  // [3*cap] ion-site forces (ions and sites)
  double *frf;                  // [nchunk_rf*3*cap] RFPAR cross partials
  int nchunk_rf, chunk_rf;
  // FP32 path.  Particle records: positions as float-float pairs (the
  // authoritative coordinates while the host marks them fresh), pair-law
  // type code and charge (written by k_pack), RFPAR data (field kernel).
  F32C f;
  float4 *pk1;                  // [cap] (x_hi, y_hi, z_hi, bits(type-1 | mobile<<16))
  float4 *pk2;                  // [cap] (x_lo, y_lo, z_lo, srfe)
  float4 *pk3;                  // [cap] (reff, q, bits(rf flags), 0), flags in fields.cu
  float4 *rfd;                  // [2*cap] srfe and reff gradients (xyz, 0)
  float *ffield_f, *fis_f;      // [3*cap] single-particle / ion-site forces
  // FP32 ion-site tiles (32 ions x 32 sites a warp): ion partials per site
  // tile [S][3][cap], site partials per ion tile [T][3][nsites], the PROXDIFF
  // nearest-site candidates per site tile [S][6][cap] (value, site, dist,
  // dx, dy, dz) and the first site's record [5][cap]
  float *isp_ion, *isp_site, *isp_dids, *isp_seed;
  int isp_tcap;                 // ion tiles the site partials hold
  float *fii_f, *frf_f;         // [nchunk*3*cap] partial forces
  // Newton's-third-law pair kernel: per tile pair q and side (0 = row tile,
  // 1 = column tile), per lane: (fx, fy, fz, A) and B of the RFPAR chain
  float4 *tpf;                  // [npairs][2][32]
  float *tpb;                   // [npairs][2][32]
  int ntile;                    // ion tiles of 32 (0: chunked pair kernel)
  // extension mode, FP32: cell list of the ions (cells of edge >= the cutoff,
  // so every pair within it lies in the same or a neighbouring cell)
  int nc[3], ncells;            // cells per axis, total (0: no cell list)
  float cinv[3];                // cells per Angstrom along each axis
  int *cell_n, *cell_start;     // [ncells + 1]: counts (then cursors), first slot
  int *cell_ion, *ion_cell;     // [cap]: ions by cell (ascending within a cell); an ion's cell
  const float2 *fact_f;         // [ntype+1] (fact1a, fact2a)
  const float2 *zcont_ff;       // [cntpts] crossing planes (hi, lo)
  const float *esvdw_f;         // [nttyp+1] repulsion scale per combined type
  double *epart;                // [nslot*kNTerms] block partial energies
  double *eterms;               // [kNTerms] reduced energies
  int *warn;                    // [nttyp+1]
  // ---- GRAND in float-float ----
  FFC ffc;
  const PairFF *ppff;           // [ntc]
  const float2 *cgff, *qcff;    // [ntype+1] charge, celec * charge
  const float2 *esvff;          // [nttyp+1] repulsion scale per combined type
  const float2 *bufff;          // [3*(nbuffer+1)] (avnum, mu, kb) per buffer, 1-based
  const float2 *epff;           // [3*cnt] effective-potential pieces (p1, p2, p3)
  float4 *gc_rff;               // [cap] per ion: (q srfe reff, reff^2), each hi, lo
  TrialFF *tff;                 // [kSpec] the round's trials
  double *ipart;                // [nslot*kSpec] INTERACT (per block) and GRAND
                                // (per block and attempt) partial sums
  int *ierr;                    // [nslot*kSpec] GRAND: error flags of the partials
};

}  // namespace bgpu
