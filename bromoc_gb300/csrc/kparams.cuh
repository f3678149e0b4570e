// Kernel parameter block: every kernel receives one KP by value.  Device
// pointers only; the host-side context (api.cu) owns the allocations.
#pragma once
#include "common.cuh"

namespace bgpu {

struct Grid3 {
  int nclx, ncly, nclz;
  double dcel, idcel, tranx, trany, tranz, xbcen, ybcen, zbcen;
};

struct PairParamF {  // FP32 copy of PairParam for the single-precision path
  float fct, epp4, sgp2, c0, c1, c2, c3, c4, sc0, sc1, sc2, dm2lo, dm2hi, dmi;
  int flags, nxi;
};

struct KP {
  // ---- sizes (host-known) ----
  int cap, nsites, nfix, ntype, nold, nttyp, ndna, ntc;
  DevState *st;   // live ntot, buffer counters, error flags
  // ---- system ----
  int shape, qcountion;
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
  const double *ep;       // [3*cnt] reference form (p1,p2,p3)
  const float4 *ep32;     // [cnt] local form (a, b, c, x_k)
  int cnt;
  double rth, srpx, srpk, srpy, res, ires;
  float rthf, srpxf, srpkf, srpyf, iresf;  // FP32 copies for the fast path
  // ---- sites ----
  const int *typtyp;      // [nsites] 1-based combined type
  const double *sitecharge;
  const uint8_t *stfree;
  const int *site_map;    // [nsites] nmcden map or nullptr
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
  Trial *trial;
  // ---- scratch ----
  double *ffield;               // [3*cap] single-particle field forces
  double *fii;                  // [nchunk_ii*3*cap] ion-ion partial forces
  int nchunk_ii, chunk_ii;
  double *fis;                  // [3*cap] ion-site forces (ions and sites)
  double *frf;                  // [nchunk_rf*3*cap] RFPAR cross partials
  int nchunk_rf, chunk_rf;
  double *epart;                // [nslot*kNTerms] block partial energies
  double *eterms;               // [kNTerms] reduced energies
  int *warn;                    // [nttyp+1]
  double *ipart;                // [nslot] INTERACT block partials
};

}  // namespace bgpu
