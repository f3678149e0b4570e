/*
 * bromoc_gpu.h -- C ABI of the GB300 (sm_103a) cg-gcmc-bd inner loop.
 *
 * The library replaces the hot subroutines of BROMOC's cg-gcmc-bd simulator
 * (Fortran 90, module-global state, no argument lists) with a context object
 * that holds the same state on the device.  Every entry point returns an int
 * status (BROMOC_OK == 0) and never aborts the host process; the message of
 * the last failure is available from bromoc_gpu_last_error().
 *
 * Conventions mirror the reference:
 *   - particle order: DNA sites 1..nsites, fixed ions nsites+1..nsites+nfix,
 *     mobile ions nsites+nfix+1..ntot (cg-gcmc-bd/src/energy.mono.f90:120-123);
 *   - typei(i) is the signed ion type, sign = side of cz
 *     (cg-gcmc-bd/src/grand.f90:73-74, count.f90:58-62);
 *   - units: Angstrom, ps, kcal/mol, e;  "real" == double;
 *   - pair parameter tables are indexed by the packed pair index "is" of
 *     cg-gcmc-bd/src/nindex.f90:19-35 (1-based in the tables passed here).
 *
 * Arrays passed in are host memory and are copied; the caller keeps
 * ownership.  One host thread per context.
 */
#ifndef BROMOC_GPU_H
#define BROMOC_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define BROMOC_ABI_VERSION 2

/* ---- status codes ------------------------------------------------------ */
enum {
  BROMOC_OK = 0,
  BROMOC_E_ARG = 1,      /* bad argument (null pointer, size out of range)   */
  BROMOC_E_STATE = 2,    /* call order: a required set_* call is missing      */
  BROMOC_E_CUDA = 3,     /* a CUDA runtime call failed                        */
  BROMOC_E_CAPACITY = 4, /* ntot would exceed the context capacity (datom)    */
  BROMOC_E_NOMEM = 5,    /* device allocation failed                          */
  BROMOC_E_DEVICE = 6    /* a kernel reported an error flag (e.g. bad index)  */
};

/* ---- energy term slots (grandmod.f90:56, gsbpmod.f90:173) -------------- */
enum {
  BROMOC_ENER = 0,     /* total                                            */
  BROMOC_EELEC,        /* ion-ion Coulomb                                  */
  BROMOC_EVDW,         /* ion-ion Lennard-Jones                            */
  BROMOC_ESRPMF,       /* ion-ion short-range PMF                          */
  BROMOC_EEFPOT,       /* ion-ion tabulated effective potential            */
  BROMOC_EQQMX,        /* ion-site Coulomb                                 */
  BROMOC_EVDWMX,       /* ion-site Lennard-Jones                           */
  BROMOC_ESRPMFMX,     /* ion-site short-range PMF                         */
  BROMOC_EEFPOTMX,     /* ion-site tabulated effective potential           */
  BROMOC_EMEMB,        /* membrane (membrane.f90)                          */
  BROMOC_EGSBPA,       /* static field (staticf1.f90)                      */
  BROMOC_EGSBPB,       /* reaction field (rfpar.f90 copies erfpar here)    */
  BROMOC_EVDWGD,       /* grid repulsion (vdwgd1trln/spln.f90)             */
  BROMOC_ERFPAR,       /* reaction-field parameters (rfpar.f90)            */
  /* DNA bonded and Go-like terms (nucleotmod.f90:40-48) */
  BROMOC_EBOND,        /* bond stretch                                     */
  BROMOC_EANG,         /* bond angle                                       */
  BROMOC_EDIHE,        /* torsion                                          */
  BROMOC_ESTACK,       /* native contacts (stacking)                       */
  BROMOC_EBP,          /* base-pair hydrogen bonds                         */
  BROMOC_EEX,          /* excluded volume                                  */
  BROMOC_EQQ,          /* phosphate-phosphate Coulomb / Debye-Hueckel      */
  BROMOC_ESOLV,        /* solvent-induced                                  */
  BROMOC_ECON,         /* harmonic position constraints (CONTRANS)         */
  BROMOC_NTERMS
};

/* ---- term switches (the ENERGY/INTERACT/TEST keyword masks,
 *      shell_simul.f90:1428-1465) ----------------------------------------- */
enum {
  BROMOC_M_NONBOND = 1u << 0, /* Qnonbond: ion-ion and ion-site pairs      */
  BROMOC_M_MEMB = 1u << 1,    /* Qmemb                                     */
  BROMOC_M_PHIX = 1u << 2,    /* Qphix                                     */
  BROMOC_M_PHIV = 1u << 3,    /* Qphiv                                     */
  BROMOC_M_RFPAR = 1u << 4,   /* Qrfpar                                    */
  BROMOC_M_BOND = 1u << 5,    /* Qnobond: DNA bond, angle and torsion terms */
  BROMOC_M_MMIJ = 1u << 6,    /* Qmmij: reaction field of the MMIJ basis    */
  BROMOC_M_ALL = 0x7fu
};

enum { BROMOC_BOX = 0, BROMOC_SPHERE = 1, BROMOC_ECYL = 2 };

/* FP64 mirrors the reference's -fdefault-real-8 build.  FP32 runs ENERGY and
 * the BD update in single precision: positions as float-float pairs, pair
 * laws and map gathers in FP32, compensated force sums, energy totals
 * accumulated in FP64 across blocks.  INTERACT stays FP64.  GRAND evaluates
 * its ΔE and acceptance in float-float arithmetic on the FP32 pipe (about
 * 48 bits), with the FP64 law for pairs closer than 0.1 A and the FP64
 * acceptance formula where an exponent leaves float's range. */
enum { BROMOC_FP64 = 0, BROMOC_FP32 = 1 };

/* BD update variants: dynamics0 (uniform D), dynamics1 (z-switch D,
 * DIFFUSION), dynamics2 (spline D(z), PROFILE), dynamics3 (DNA-proximity D,
 * PROXDIFF) -- simul1.f90:369-379. */
enum { BROMOC_DYN0 = 0, BROMOC_DYN1 = 1, BROMOC_DYN2 = 2, BROMOC_DYN3 = 3 };

/* ---- parameter blocks --------------------------------------------------- */

/* SYSTEM + SIMUL scalars: shell_simul.f90:782-947, 1198-1413. */
typedef struct bromoc_system {
  int32_t shape;         /* BROMOC_BOX / BROMOC_SPHERE / BROMOC_ECYL          */
  int32_t qcountion;     /* count z-plane crossings (countions.f90)           */
  double lx, ly, lz;     /* box edges, or ellipse diameters + length (ECYL)   */
  double cx, cy, cz;     /* system centre                                     */
  double rsphe;          /* sphere radius (SPHERE)                            */
  double temp;           /* K                                                 */
  double kbt;            /* kcal/mol: kboltz*temp/kcalmol (shell_simul:865)   */
  double cdie;           /* solvent dielectric                                */
  double dt;             /* ps                                                */
  double bdmax;          /* per-component BD displacement clamp (Angstrom)    */
} bromoc_system;

/* Ion types (PARTICLES) and combined types (reasig.f90). */
typedef struct bromoc_types {
  int32_t ntype;             /* typei values are +-[nold+1, ntype]           */
  int32_t nold;              /* types defined before PARTICLES (DNA)         */
  int32_t nttyp;             /* combined types: DNA site types + ion types   */
  int32_t ndna;              /* combined types 1..ndna are DNA site types    */
  const int32_t *nwtype;     /* [ntype] ion type -> combined type (1-based)  */
  const double *cg;          /* [ntype] charge (e)                           */
  const double *diffusion;   /* [ntype] diffusion constant (A^2/ps)          */
} bromoc_types;

/* Pair laws: Coulomb (fct), LJ 12-6 (epp4, sgp2), SRPMF (c0..c4) and the
 * tabulated effective potential (efpmod).  All arrays indexed by "is". */
typedef struct bromoc_pairs {
  int32_t ntc;               /* number of packed pair indices               */
  const uint8_t *qchr, *qlj, *qsrpmf, *qefpot;   /* [ntc] law switches       */
  const double *fct;         /* [ntc] celec*qi*qj/cdie                       */
  const double *epp4;        /* [ntc] 4*eps                                  */
  const double *sgp2;        /* [ntc] sigma^2                                */
  const double *c0, *c1, *c2, *c3, *c4; /* [ntc] SRPMF, c2 already 1/c2      */
  double rth;                /* SRPMF cutoff SQUARED (shell_simul:1686)     */
  double srpx, srpk, srpy;   /* SRPMF taper (shell_simul:1683-1685)         */
  /* tabulated effective potential (efpmod.f90, polynom.f90:172-254) */
  int32_t cnt;               /* number of quadratic pieces                   */
  const double *ep;          /* [3*cnt] (p1,p2,p3) of piece k at ep[3k..]    */
  const double *sc;          /* [3*ntc] core a/r^12+b and tail a/r^6 consts  */
  const double *dm2;         /* [2*ntc] (mindist^2, maxdist^2)               */
  const double *dmi;         /* [ntc] mindist                                */
  const int32_t *nxi;        /* [ntc] 1-based first piece of the pair        */
  double res;                /* table spacing                                */
} bromoc_pairs;

/* DNA interaction sites (NUCLEOTIDES). */
typedef struct bromoc_sites {
  int32_t nsites;
  const int32_t *typtyp;     /* [nsites] combined type 1..ndna               */
  const double *charge;      /* [nsites] cgnuc for 'P' sites, else 0         */
  const uint8_t *stfree;     /* [nsites] site moves (not FIXSITE)            */
  const int32_t *phiv_map;   /* [nsites] nmcden repulsion map, or NULL       */
} bromoc_sites;

/* DNA bonded and Go-like terms between sites (nucleotmod.f90; the lists of
 * bonds.f90, angles.f90, dihedral.f90 and go_qq.f90, the forms of
 * energy.mono.f90:196-582).  Site numbers are 1-based; a term's sites are
 * consecutive (sitebond[2k], sitebond[2k+1] are term k's two sites: the
 * Fortran sitebond(k,1), sitebond(k,2)).  A count of 0 allows a NULL list.
 *   bond      eps (d-d0)^2 (1 + 100 (d-d0)^2)
 *   angle     700 eps (theta-theta0)^2
 *   torsion   28 eps (1 - cos(phi-phi0))
 *   stack     4 eps ((sg/d)^12 - (sg/d)^6)
 *   base pair eps_bp (sg/d)^10 (20 (sg/d)^2 - 24), eps_bp = 2.532 eps s
 *             for G-C (bpgc != 0) and 2 eps s otherwise, s = scalepairing
 *   excluded  4 eps ((sg/d)^12 - (sg/d)^6) + eps for d < sg
 *   qq        fctn/d, or fctn e^{-d/kappa}/d (qdeby 1, or qdeby 2 with both
 *             sites outside the system, grandmod.f90:74-98)
 *   solvent   epsolv (1 - e^{0.1875 (13.38-d)})^2 - epsolv
 * Constant applied forces (APFOR) act on free sites; CONTRANS adds
 * harmonic springs on single sites or on the sites' centre (csn 0). */
typedef struct bromoc_nucleotides {
  double epsnuc;             /* energy scale eps (kcal/mol)                  */
  double scalepairing;       /* base-pair scale s                            */
  double fctn;               /* celec cgnuc^2 / cdie                         */
  double kappa;              /* Debye length (A), qdeby != 0                 */
  int32_t qdeby;             /* 0 Coulomb, 1 Debye-Hueckel, 2 hybrid         */
  int32_t qsolv;             /* solvent-induced S-S terms                    */
  double epsolv;
  int32_t nbond;   const int32_t *sitebond;  const double *distbond; /* d0 */
  int32_t nangle;  const int32_t *siteangle; const double *valangle; /* rad, */
                                             /* middle site is the vertex  */
  int32_t ndihe;   const int32_t *sitedihe;  const double *valdihe;  /* rad */
  int32_t nstack;  const int32_t *sitestack; const double *sgstack;
  int32_t nbp;     const int32_t *sitebp;    const double *sgbp;
  const uint8_t *bpgc;       /* [nbp] first site is a G or C base            */
  int32_t nex;     const int32_t *siteex;    const double *sgex;
  int32_t nqq;     const int32_t *siteqq;
  int32_t nsolv;   const int32_t *siteslv;
  int32_t afn;     const int32_t *sn;        /* APFOR sites                  */
  const double *af;          /* [3*afn] force on site sn[k] (kcal/mol/A)     */
  int32_t ctn;               /* CONTRANS entries                             */
  const int32_t *csn;        /* [ctn] site, or 0 for the sites' centre       */
  const double *kx, *ky, *kz;          /* [ctn] spring constants             */
  const double *contrx, *contry, *contrz; /* [ctn+1] anchors; entry ctn is  */
                                       /* the second strand's centre (unsplit) */
  int32_t qunsplit;          /* centre springs per strand (two strands)      */
  int32_t nsites1st;         /* sites of the first strand                    */
  /* NOTRAN (simul1.f90:380-385): after every BD step the sites' centre
   * along each flagged axis is put back to notr (x - sum(x)/nsites + notr) */
  int32_t qnotr[3];
  double notr[3];
} bromoc_nucleotides;

/* Reaction field of the MMIJ basis (GSBP mmij keywords,
 * shell_simul.f90:2780-2830, and the file readmmij.f90 reads).  RECTBOX:
 * Legendre products P_a(2x/wx) P_b(2y/wy) P_c(2z/wz) over the region
 * |x| <= wx/2, |y| <= wy/2, |z| <= wz/2 (the widths wx = rbxmax - rbxmin
 * ...; the region is centred at the origin as in the reference), basis
 * orders lstpx/lstpy/lstpz, energy scale rfscal.  SPHERE: the multipoles
 * r^l P_l^m(cos theta) {cos, sin}(m phi), l < nmpol <= 25, inside radius
 * srdist.  mmij: ntpol x ntpol, row-major as in the file; the lower
 * triangle is taken from the upper one (readmmij.f90). */
typedef struct bromoc_mmij {
  int32_t shape;             /* BROMOC_BOX (RECTBOX) or BROMOC_SPHERE        */
  int32_t xnpol, ynpol, znpol;                  /* RECTBOX                   */
  const int32_t *lstpx, *lstpy, *lstpz;         /* [ntpol] orders            */
  double rbxmin, rbxmax, rbymin, rbymax, rbzmin, rbzmax;
  double rfscal;
  int32_t nmpol;             /* SPHERE: ntpol = nmpol^2                     */
  double srdist;
  const double *mmij;        /* [ntpol*ntpol]                                */
} bromoc_mmij;

/* Grid header of a PB map file: readphi.f90:43-52 (z fastest, x slowest). */
typedef struct bromoc_grid {
  int32_t nclx, ncly, nclz;
  double dcel;
  double xbcen, ybcen, zbcen;
} bromoc_grid;

/* Repulsion map options: GSBP phiv keywords, shell_simul.f90:2703-2777. */
typedef struct bromoc_phiv_opts {
  int32_t nmaps;             /* 1, or one map per type under nmcden          */
  int32_t trilinear;         /* 1 = vdwgd*trln, 0 = vdwgd*spln (bspline)     */
  int32_t nmcden;            /* per-type maps                                */
  double svdw, vzmin, vzmax, thold8, thold27;
  const int32_t *map_of_type;/* [ntype] 0-based map per ion type (nmcden)   */
  const double *scal;        /* [nttyp] SVDW scale per combined type or NULL */
} bromoc_phiv_opts;

/* Membrane (MEMBRANE + SYSTEM volt/ionic), shell_simul.f90:1563-1669. */
typedef struct bromoc_membrane {
  int32_t qpore;
  double voltage;            /* kcal/mol/e (volt*Coulomb/kcalmol)            */
  double afact, ikappa, ceps, zmemb1, zmemb2;
  const double *ampl1;       /* [nttyp]                                      */
  const double *p1;          /* [2*nttyp] (pmemb, 1/pmemb)                   */
  const double *ampl2;       /* [nttyp]                                      */
  const double *p2;          /* [2*nttyp] (ppore, 1/ppore)                   */
  const double *rcylinder;   /* [nttyp]                                      */
} bromoc_membrane;

/* Space-dependent diffusion models and DNA-site BD factors. */
typedef struct bromoc_diffusion {
  double plength2, pcenter;  /* DIFFUSION: half pore length, pore centre     */
  const double *ampl3;       /* [ntype] lowfraction                          */
  const double *p3;          /* [ntype] switchlength                         */
  int32_t nspline;           /* PROFILE cubic spline D(z)/D0                 */
  const double *xs, *ys, *b, *c, *d;
  double diff0, ibeta, diffcutoff;   /* PROXDIFF                             */
  double fact0n1, fact0n2;   /* DNA sites: diffnuc*kbtdna*dt, sqrt(2 dt D)   */
  int32_t qdnafree;          /* DNA not clamped to the system               */
} bromoc_diffusion;

/* GCMC buffers (BUFFERS), grandmod.f90:41-47. */
typedef struct bromoc_buffers {
  int32_t nbuffer;
  const int32_t *ibfftyp;    /* [nbuffer] ion type                           */
  const double *avnum, *mu, *kb, *lzmin, *lzmax, *rmin, *rmax;
  const uint8_t *qbufferbias;
  const int32_t *nat;        /* [nbuffer] ions currently in the buffer       */
  const int32_t *ntotat;     /* [nbuffer] running total used by kb bias      */
} bromoc_buffers;

typedef struct bromoc_ctx bromoc_ctx;

/* ---- context -------------------------------------------------------------
 * capacity: maximum ntot (the reference's static datom = 23000,
 *           grandmod.f90:24); precision: BROMOC_FP64 or BROMOC_FP32;
 * stream:   cudaStream_t to launch on (NULL = a stream owned by the ctx).   */
int bromoc_gpu_create(int32_t capacity, int32_t precision, void *stream,
                      bromoc_ctx **out);
int bromoc_gpu_destroy(bromoc_ctx *ctx);
const char *bromoc_gpu_last_error(const bromoc_ctx *ctx);
int bromoc_gpu_abi_version(void);

/* ---- module state (replaces the deck-time fills of the Fortran modules) */
int bromoc_gpu_set_system(bromoc_ctx *ctx, const bromoc_system *sys);
int bromoc_gpu_set_types(bromoc_ctx *ctx, const bromoc_types *types);
int bromoc_gpu_set_pairs(bromoc_ctx *ctx, const bromoc_pairs *pairs);
int bromoc_gpu_set_sites(bromoc_ctx *ctx, const bromoc_sites *sites);
/* DNA bonded and Go-like term lists (after set_sites; NULL clears them).
 * ENERGY adds them to the site forces and to ener; INTERACT of a site adds
 * the terms that involve it (interact.f90:211-334, with its base-pair
 * scale of 1). */
int bromoc_gpu_set_nucleotides(bromoc_ctx *ctx, const bromoc_nucleotides *nuc);
/* MMIJ reaction field (NULL switches it off).  ENERGY adds egsbpb
 * (rect_rf1.f90 / sphe_rf1.f90) to ener and its forces to the mobile ions
 * in the region; INTERACT of a mobile ion adds E(coef) - E(coef without it)
 * (rect_rf0.f90 / sphe_rf0.f90).  GRAND refuses a system with it on
 * (BROMOC_E_STATE). */
int bromoc_gpu_set_mmij(bromoc_ctx *ctx, const bromoc_mmij *m);
/* static field phix (readphi PHIX, gsbpmod phix) -- staticf1/staticf0 */
int bromoc_gpu_set_phix(bromoc_ctx *ctx, const bromoc_grid *g,
                        const float *phix);
/* repulsion map phiv after binarisation and repwalls (values 0..127) */
int bromoc_gpu_set_phiv(bromoc_ctx *ctx, const bromoc_grid *g,
                        const int8_t *phiv, const bromoc_phiv_opts *opts);
/* reaction-field parameter grids gsrfen/greff (readrfpar, rfpar.f90:373) */
int bromoc_gpu_set_rfpar(bromoc_ctx *ctx, const bromoc_grid *g, int32_t nmaps,
                         const float *gsrfen, const float *greff,
                         double reffac, const int32_t *map_of_type);
int bromoc_gpu_set_membrane(bromoc_ctx *ctx, const bromoc_membrane *m);
int bromoc_gpu_set_diffusion(bromoc_ctx *ctx, const bromoc_diffusion *d);
int bromoc_gpu_set_countions(bromoc_ctx *ctx, int32_t cntpts,
                             const double *zcont);
int bromoc_gpu_set_buffers(bromoc_ctx *ctx, const bromoc_buffers *b);

/* ---- particles (grandmod x,y,z,typei,ibuffer) ------------------------- */
int bromoc_gpu_set_particles(bromoc_ctx *ctx, int32_t ntot, int32_t nsites,
                             int32_t nfix, const double *x, const double *y,
                             const double *z, const int32_t *typei,
                             const int32_t *ibuffer);
int bromoc_gpu_get_particles(bromoc_ctx *ctx, int32_t *ntot, double *x,
                             double *y, double *z, int32_t *typei,
                             int32_t *ibuffer);

/* ---- hot path ------------------------------------------------------------
 * ENERGY (energy.mono.f90:19-692 minus DNA bonded terms): total energy with
 * the term breakdown in eterms[BROMOC_NTERMS]; forces into fx/fy/fz (host,
 * may be NULL) when qforces != 0 -- they receive the CURRENT device ntot
 * values, which GCMC may have raised above the last upload, so pass
 * capacity-sized buffers (the reference's datom-sized arrays); warn[nttyp]
 * (may be NULL) receives the "particle inside membrane or protein"
 * counters. */
int bromoc_gpu_energy(bromoc_ctx *ctx, uint32_t terms, int32_t qforces,
                      double *fx, double *fy, double *fz, double *eterms,
                      int32_t *warn);

/* INTERACT (interact.f90:19-419): FP64 energy of particle j (1-based; j ==
 * ntot+1 is an insertion trial) of combined-or-ion type jtype placed at
 * (xj,yj,zj) with the rest of the system. */
int bromoc_gpu_interact(bromoc_ctx *ctx, uint32_t terms, double xj, double yj,
                        double zj, int32_t jtype, int32_t j, double *dener);

/* One BD update with the forces of the last bromoc_gpu_energy(qforces)
 * call: dynamics{0,1,2,3} on the mobile ions, dynamics0nuc on free DNA
 * sites, fixcoor, countions.  Noise is Philox4x32-10 keyed by
 * (seed, step, particle slot, component). */
int bromoc_gpu_dynamics(bromoc_ctx *ctx, int32_t variant, uint64_t seed,
                        uint64_t step);

/* nsteps x (ENERGY with forces + BD update), device resident; steps are
 * numbered step0, step0+1, ... for the noise stream.  eterms (may be NULL)
 * receives the energy of the last step's ENERGY call. */
int bromoc_gpu_bd_steps(bromoc_ctx *ctx, uint32_t terms, int32_t variant,
                        int32_t nsteps, uint64_t seed, uint64_t step0,
                        double *eterms);

/* Drop-in for simul1.f90's BD loop over HOST arrays: uploads x,y,z,typei,
 * runs nsteps, downloads x,y,z (the arrays are updated in place). */
int bromoc_gpu_bd_steps_host(bromoc_ctx *ctx, uint32_t terms, int32_t variant,
                             int32_t nsteps, uint64_t seed, uint64_t step0,
                             int32_t ntot, int32_t nsites, int32_t nfix,
                             double *x, double *y, double *z,
                             const int32_t *typei, double *eterms);

/* Drop-in for one or more cycles of simul1.f90:351-390 over HOST arrays:
 * per cycle GRAND(ngcmc) then nbd x (ENERGY with forces + DYNAMICSn).  The
 * particle arrays (capacity-sized buffers) are uploaded, advanced on the
 * device and written back with the new *ntot (GCMC changes it); entries
 * past the new *ntot may be overwritten too (up to *ntot + ncycle*ngcmc).
 * Cycles are numbered cycle0, cycle0+1, ...; BD steps
 * (cycle-1)*nbd + istep - 1.  Each cycle ends with COUNT (and, when
 * switched on, a profile sample), as simul1.f90 does.  The work is queued in
 * stream order with one wait at the end: the call returns when the arrays
 * hold the result. */
int bromoc_gpu_simul_cycles_host(bromoc_ctx *ctx, uint32_t terms,
                                 int32_t variant, int32_t ncycle,
                                 int32_t ngcmc, int32_t nbd, uint64_t seed,
                                 uint64_t cycle0, int32_t *ntot,
                                 int32_t nsites, int32_t nfix, double *x,
                                 double *y, double *z, int32_t *typei,
                                 int32_t *ibuffer, double *eterms);

/* Ion-ion pair energy and forces for callers that must not allocate device
 * memory while they run -- e.g. a host program that reserves its whole GPU
 * memory budget at start-up and treats any later allocation as a failure,
 * or an embedding whose device allocator belongs to another runtime.  It
 * has no counterpart in the reference.
 *
 * Inputs and outputs are caller-owned DEVICE buffers: x,y,z,typei [n] (ions
 * only, the first nfix fixed; typei signed ion types), fx,fy,fz [n] and
 * eterms4 [4] = (eelec, evdw, esrpmf, eefpot).  The pair laws come from ctx
 * (set_system/set_types/set_pairs; its precision selects FP64 or FP32 pair
 * arithmetic); results equal bromoc_gpu_energy with BROMOC_M_NONBOND on a
 * system without sites.  The scratch is a static device array sized for at
 * most 4096 ions (about 1.6 MB per device, held until the process exits);
 * n > 4096 returns BROMOC_E_CAPACITY.  No allocation or free happens in the
 * call.  All calls on a device share that scratch: calls that overlap on
 * the GPU race.  The first call on a device resolves the scratch address
 * (cudaGetSymbolAddress with that device current) and keeps it for the life
 * of the process -- make that first call before any stream capture; after a
 * device reset the library is not used again in the process.  Each call waits
 * on its stream before it returns (it reads back an error word), so the
 * results are written when it returns and no call can be made inside a
 * stream capture; n == 0 writes zero energies (the
 * per-ion arrays may then be null). */
int bromoc_gpu_pair_energy_static(bromoc_ctx *ctx, int32_t n, int32_t nfix,
                                  const double *x, const double *y,
                                  const double *z, const int32_t *typei,
                                  double *fx, double *fy, double *fz,
                                  double *eterms4);

/* Number of kernels this context has launched so far. */
int64_t bromoc_gpu_launch_count(const bromoc_ctx *ctx);
/* The live particle count as the context's stream reaches this call, copied
 * to *dst (pinned host memory) without waiting: valid once the stream has
 * synchronised.  A driver that records the count every cycle need not stop
 * the GPU.  No counterpart in the reference (its count is a host global). */
int bromoc_gpu_live_count_async(bromoc_ctx *ctx, int32_t *dst);

/* ---- diagnostics (no counterpart in the reference) ----------------------
 * Per-kernel timing with CUDA events recorded on the launching stream around
 * every launch of the kernel family `which` while timing is on. */
enum {
  BROMOC_K_PAIRS = 0,    /* ion-ion pair kernel                            */
  BROMOC_K_RFCROSS = 1,  /* RFPAR cross-term pair kernel                   */
  BROMOC_K_FIELDS = 2,   /* single-particle map/membrane kernel            */
  BROMOC_K_ASSEMBLE = 3, /* force assembly + BD update                     */
  BROMOC_K_LOOP = 4,     /* fused BD loop (all of the above, many steps)   */
  BROMOC_K_GRAND = 5,    /* GRAND (all attempts of a call)                 */
  BROMOC_K_NKINDS = 6
};
int bromoc_gpu_kernel_timing(bromoc_ctx *ctx, int32_t on);
/* bd_steps in FP32 mode runs the steps of a system without sites as one
 * cooperative launch (on = 1, the default) or one launch per kernel and
 * step (on = 0); the trajectories agree.  No counterpart in the reference. */
int bromoc_gpu_set_fused_bd(bromoc_ctx *ctx, int32_t on);
/* Extension mode, no counterpart in the reference: a periodic box system
 * (after set_system with BROMOC_BOX) whose ion pairs interact through the
 * nearest periodic image when closer than rcut (Angstrom; plain cutoff, no
 * shift), with every move wrapped into the box instead of clamped.  Ions
 * only (no sites), without RFPAR; in FP32 mode up to 8192 ions.  on = 0
 * returns to the reference's hard walls without cutoff. */
int bromoc_gpu_set_periodic(bromoc_ctx *ctx, int32_t on, double rcut);
/* total milliseconds and number of timed launches since timing was turned
 * on (synchronises the context's stream) */
int bromoc_gpu_kernel_time(bromoc_ctx *ctx, int32_t which, double *total_ms,
                           int64_t *launches);
/* Self-test of the bounded waits of the cooperative kernels (no counterpart
 * in the reference): one block waits, through the grid barrier's own wait
 * limited to `spins` polls, for an arrival that a second block makes only
 * when `arrive` is nonzero.  *err_word receives the device error word: 16
 * (the barrier flag) when the wait ran out, 0 when the arrival came.  The
 * kernel returns either way; synchronous, on the current device. */
int bromoc_gpu_wait_selftest(int32_t spins, int32_t arrive, int32_t *err_word);
/* Measured FP32 FMA throughput of the current device (TFLOP/s), the
 * denominator of the pair kernels' roofline. */
int bromoc_gpu_fp32_peak(void *stream, double *tflops);
/* Accuracy check of the float-float arithmetic GRAND evaluates its ΔE in
 * (no counterpart in the reference): out[i] = f(x[i]) for the function
 * fn below (binary ones take x[i] and x[(i+1) mod n]), each input first
 * rounded to float-float, on the current device (synchronous). */
enum {
  BROMOC_FF_EXP = 0,
  BROMOC_FF_COS = 1,
  BROMOC_FF_SQRT = 2,
  BROMOC_FF_RCP = 3,
  BROMOC_FF_MUL = 4,
  BROMOC_FF_DIV = 5,
  BROMOC_FF_ADD = 6,
  BROMOC_FF_RSQRT = 7
};
int bromoc_gpu_ff_check(int32_t fn, int32_t n, const double *x, double *out);

/* GRAND (grand.f90:19-121): ngcmc grand-canonical insertion/deletion
 * attempts of cycle `cycle` (1-based icycle), device resident.  Uniforms are
 * Philox4x32-10 keyed by (seed, cycle, attempt, draw).  dener_sum (may be
 * NULL) receives the accumulated energy change (ener += dener). */
int bromoc_gpu_grand(bromoc_ctx *ctx, uint32_t terms, int32_t ngcmc,
                     uint64_t seed, uint64_t cycle, double *dener_sum);
/* Buffer counters after GRAND: nat, ninsert, nremove [nbuffer] and the
 * occupancy histogram prob[nbuffer*(capacity+1)] (prob(ib,n) of simul1). */
/* METROPOLIS (metropolis.f90:31-55, move.f90:19-45): nmcm Monte Carlo moves
 * of cycle `cycle`, device resident.  Each picks a mobile ion and a
 * displacement of up to mcmax/2 per axis (drawn again while the position
 * lies outside the system, at most 1000 times; then the move is skipped),
 * evaluates INTERACT at the old and the new position, and accepts downhill
 * moves and uphill ones with probability exp(-(enew - eold)/kT).  Uniforms:
 * Philox4x32-10 keyed by (seed, cycle, move, draw) under their own stream
 * tag.  naccept, dener_sum (may be NULL): accepted moves and their summed
 * energy change (ener += dener).  Systems with fixed ions are refused. */
int bromoc_gpu_metropolis(bromoc_ctx *ctx, uint32_t terms, int32_t nmcm, double mcmax,
                          uint64_t seed, uint64_t cycle, int32_t *naccept,
                          double *dener_sum);
int bromoc_gpu_get_buffers(bromoc_ctx *ctx, int32_t *nat, int32_t *ninsert,
                           int32_t *nremove, int32_t *prob);
/* countions crossing counters [(ntype-nold)*cntpts], type-major */
int bromoc_gpu_get_countions(bromoc_ctx *ctx, int32_t *nforward,
                             int32_t *nbackward);

/* Per-particle PROXDIFF nearest-site record dids(5,ntot) of the last
 * ENERGY call (energy.mono.f90:603-621), 5 doubles per particle. */
int bromoc_gpu_get_dids(bromoc_ctx *ctx, double *dids);

/* COUNT (count.f90:19-95; simul1.f90:462 calls it once a cycle, after the
 * BD steps): each mobile ion's buffer from its position, nat, the sign of a
 * buffer ion's type by its side of cz, then ntotat += nat.  Queued without
 * a wait; a buffer ion outside the system is reported as BROMOC_E_DEVICE by
 * the next call that reads the device flags.  No-op without buffers.
 * bromoc_gpu_simul_cycles_host runs it every cycle. */
int bromoc_gpu_count(bromoc_ctx *ctx);
/* ntotat of every buffer (the running sum of nat that the kb bias uses). */
int bromoc_gpu_get_ntotat(bromoc_ctx *ctx, int32_t *ntotat);

/* ---- per-cycle analysis (simul1.f90:176-188, 476-509) ---------------------
 * Switch the z-density profile of the mobile ions (qrho, RHO), of the DNA
 * sites (qrdna, RHDNA) and the radial distribution of the mobile ions
 * around particle igr (1-based; qgr, RDF, shells of dr, npoints of them),
 * and clear their counts.  z bins as the reference: from the system's lower
 * z face, 0.5 A wide, nzmax = min(int(2 lz), npoints).  A particle below
 * the first bin is not counted (the reference writes outside its array). */
int bromoc_gpu_set_profiles(bromoc_ctx *ctx, int32_t qrho, int32_t qrdna,
                            int32_t qgr, int32_t igr, double dr,
                            int32_t npoints);
/* One sample from the current state, queued without a wait
 * (bromoc_gpu_simul_cycles_host takes one per cycle itself). */
int bromoc_gpu_accum_profiles(bromoc_ctx *ctx);
/* The sums so far (counts, as the reference's sums of 1.0); any output may
 * be NULL: rho[(itype-nold-1)*nzmax + iz-1], rdna[(typtyp-1)*nzmax + iz-1],
 * gr[(itype-nold-1)*npoints + ir-1], the bin count and the RDF's irmax. */
int bromoc_gpu_get_profiles(bromoc_ctx *ctx, double *rho, double *rdna,
                            double *gr, int32_t *nzmax, int32_t *irmax);

/* ---- trajectory (.btr: simul1.f90:283-287, wrttraj.f90:33-38) -------------
 * The bytes of gfortran unformatted sequential records, each framed by
 * 4-byte length markers, for the caller to append to the file.  With
 * buf == NULL only *nbytes is set (the size needed).
 * Header: nframe, nttyp, atnam2(1:nttyp) (character*4 each). */
int bromoc_gpu_traj_header(int32_t nframe, int32_t nttyp, const char *atnam,
                           void *buf, int64_t cap, int64_t *nbytes);
/* One frame of the current state, packed on the device: runtime (real*8),
 * ntot, typtyp(1:ntot) (ions: nwtype(|typei|)), then x, y and z rounded to
 * single precision (sng).  60 + 16 ntot bytes. */
int bromoc_gpu_traj_frame(bromoc_ctx *ctx, double runtime, void *buf,
                          int64_t cap, int64_t *nbytes);

/* ---- effective-potential table build (setup; polynom.f90, splinepot.f90,
 * discretize.f90).  Host-side C++; writes the quadratic pieces of one pair
 * into ep[3*n] and the core/tail constants into sc3[3], dm2o[2], dmio. ---- */
/* from a read table of n knots (r_k, U_k) (splinepot.f90:19-96) */
int bromoc_gpu_efpot_from_knots(int32_t n, const double *xx, const double *yy,
                                double fct, int32_t qchr, double *ep,
                                double *sc3, double *dm2o, double *dmio);

/* ---- replica batches (no reference counterpart: the reference runs one
 * system per process) --------------------------------------------------------
 * nrep independent ion systems (capacity[r] ions each) that share the FP32
 * prototype context's types, pair laws and grid maps, each with its own box,
 * particles and noise seed.  Restrictions: analytic ion-ion laws (no EFPOT),
 * at most 16 ion types, no sites or fixed ions, dynamics0, every replica
 * with the prototype's dt, kbt and bdmax.  The prototype must outlive the
 * batch.  A replica's trajectory with seed s is that of a single context
 * driven by bromoc_gpu_bd_steps with seed s (up to FP32 summation order). */
typedef struct bromoc_batch bromoc_batch;
int bromoc_batch_create(bromoc_ctx *proto, int32_t nrep, const int32_t *capacity,
                        bromoc_batch **out);
int bromoc_batch_destroy(bromoc_batch *b);
const char *bromoc_batch_last_error(const bromoc_batch *b);
/* per-replica SYSTEM blocks: box/shape for fixcoor; dt, kbt, bdmax checked */
int bromoc_batch_set_systems(bromoc_batch *b, const bromoc_system *sys);
/* GCMC buffers of replica r (grand.f90 with the prototype's ion types):
 * 1..8 buffers, the geometry in the replica's own coordinates, their
 * counts, and ibuffer[n] the buffer of each of its ions (0 none).  A later
 * set_particles of r clears its ibuffer. */
int bromoc_batch_set_buffers(bromoc_batch *b, int32_t r, const bromoc_buffers *buf,
                             const int32_t *ibuffer);
/* ngcmc GCMC attempts on every replica (grand.f90:19-121): one launch, a
 * block per replica, the attempts in order with FP64 ΔE (INTERACT on the
 * replica's records).  Replica r draws from seeds[r] with the single
 * context's counters, so it makes the moves bromoc_gpu_grand would make on
 * a context holding it.  dener[r] (optional): the summed ΔE of its accepted
 * moves.  Waits for the result; the replicas' counts then drive the next
 * bd_steps (the work lists follow them; the pair-kernel tuning stands).
 * Deletion warnings are not counted in a batch; ntotat stays as set. */
int bromoc_batch_grand(bromoc_batch *b, uint32_t terms, int32_t ngcmc,
                       const uint64_t *seeds, uint64_t cycle, double *dener);
/* COUNT (count.f90) on every replica with buffers: buffer tags, nat, type
 * signs, ntotat += nat (one launch; waits). */
int bromoc_batch_count(bromoc_batch *b);
/* Replica r's buffer counters and its ions' signed types and buffers
 * (typei/ibuffer: its current count of entries; NULL skips). */
int bromoc_batch_get_buffers(bromoc_batch *b, int32_t r, int32_t *nat, int32_t *ninsert,
                             int32_t *nremove, int32_t *typei, int32_t *ibuffer);
int bromoc_batch_set_particles(bromoc_batch *b, int32_t r, int32_t n, const double *x,
                               const double *y, const double *z, const int32_t *typei);
int bromoc_batch_get_particles(bromoc_batch *b, int32_t r, int32_t *n, double *x,
                               double *y, double *z);
/* nsteps x (ENERGY + dynamics0) of every replica; seeds[nrep]; eterms
 * (nrep x BROMOC_NTERMS, or NULL) receives the last step's energies */
int bromoc_batch_bd_steps(bromoc_batch *b, uint32_t terms, int32_t nsteps,
                          const uint64_t *seeds, uint64_t step0, double *eterms);
/* ENERGY of every replica; forces (3 doubles per slot, or NULL): replica
 * r's ion k at slot bromoc_batch_offset(b, r) + k.  Allocates a scratch
 * buffer when forces are requested. */
int bromoc_batch_energy(bromoc_batch *b, uint32_t terms, double *forces, double *eterms);
int bromoc_batch_offset(const bromoc_batch *b, int32_t r);
int bromoc_batch_slots(const bromoc_batch *b);
int64_t bromoc_batch_launch_count(const bromoc_batch *b);
/* Runs of BD steps replayed from a CUDA graph (on, the default: the seeds'
 * and step index's uploads and every step's launches captured once per
 * step count and replayed, one graph launch per call) or launched one by
 * one (off); the trajectories agree bit for bit.  No counterpart in the
 * reference, which has no batch. */
int bromoc_batch_set_graph(bromoc_batch *b, int32_t on);
/* The autotuner's state per replica size bucket (fewer than 1000 ions,
 * 1000-4000, more): warps[3] the pair kernel's chosen warps per block (0
 * when the bucket is empty or not tuned yet), items[3] its tile pairs,
 * ms[9] the measured time of one pair pass of bucket k with 2, 4, 8 warps
 * per block at ms[3k..3k+2].  Tuning runs at the first BD step after the
 * replicas' particles change.  No counterpart in the reference. */
int bromoc_batch_tuning(const bromoc_batch *b, int32_t *warps, int32_t *items, double *ms);
/* Graph launches so far (one per bd_steps call on the graph path). */
int64_t bromoc_batch_graph_launches(const bromoc_batch *b);

/* ---- adjoint of a BD segment (no reference counterpart) ----------------------
 * Gradient of a function of the segment's pair-distance histogram with respect
 * to the tabulated (EFPOT) ion-ion laws.  The prototype context supplies the
 * types, the pair tables (every ion-ion law tabulated), the box (BROMOC_BOX,
 * hard walls) and dt/kbt; ions only, at most 4 ion types, dynamics0 with the
 * Philox noise of (seed, step).  precision: arithmetic of the pair terms
 * (BROMOC_FP32 needs an FP32 prototype).  The histogram is the Gaussian-
 * smoothed pair-distance histogram, H_b = sum over the configurations after
 * each step and over pairs of K(r0 + b dr - r_ij), K the normal density of
 * width sigma, per ion-type pair (a <= b): ntp = nt (nt + 1) / 2 rows of
 * nbins.  backward takes dL/dH and returns dL/d(table parameters)
 * in the layouts of bromoc_pairs: g_ep[3 cnt] (p1, p2, p3 per piece), g_sc[3 ntc]
 * (core a/r^12 constant, core offset, tail a/r^6 constant). */
typedef struct bromoc_adj bromoc_adj;
int bromoc_adj_create(bromoc_ctx *proto, int32_t capacity, int32_t precision,
                      bromoc_adj **out);
int bromoc_adj_destroy(bromoc_adj *a);
const char *bromoc_adj_last_error(const bromoc_adj *a);
int bromoc_adj_set_particles(bromoc_adj *a, int32_t n, const double *x, const double *y,
                             const double *z, const int32_t *typei);
/* nsteps BD steps from the configuration of set_particles, checkpoints every
 * ckpt steps; hist[ntp * nbins] receives the histogram */
int bromoc_adj_forward(bromoc_adj *a, int32_t nsteps, int32_t ckpt, uint64_t seed,
                       uint64_t step0, int32_t nbins, double r0, double dr, double sigma,
                       double *hist);
int bromoc_adj_backward(bromoc_adj *a, const double *dl_dhist, double *g_ep, double *g_sc);
/* which = 0: the initial configuration, 1: the last forward run's final one */
int bromoc_adj_get_particles(bromoc_adj *a, int32_t which, double *x, double *y,
                             double *z);

#ifdef __cplusplus
}
#endif

#endif /* BROMOC_GPU_H */
