// ORACLE -- test infrastructure only (see ref_state.h).
// C API: copies the inputs into the module-like State (1-based arrays).
#include <cmath>
#include <cstring>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "bromoc_oracle.h"
#include "ref_state.h"

using bref::State;

struct bromoc_ref {
  State s;
};

namespace {
template <class T>
std::vector<T> one_based(const T *p, int n) {
  std::vector<T> v(n + 1, T());
  if (p)
    for (int i = 0; i < n; ++i) v[i + 1] = p[i];
  return v;
}
int fail(bromoc_ref *r, const char *msg, int code = BROMOC_E_ARG) {
  if (r) r->s.err = msg;
  return code;
}
}  // namespace

extern "C" {

int bromoc_ref_create(int32_t capacity, bromoc_ref **out) {
  if (!out || capacity <= 0) return BROMOC_E_ARG;
  bromoc_ref *r = new bromoc_ref();
  r->s.resize_particles(capacity);
  *out = r;
  return BROMOC_OK;
}

int bromoc_ref_destroy(bromoc_ref *r) {
  delete r;
  return BROMOC_OK;
}

const char *bromoc_ref_last_error(const bromoc_ref *r) {
  return r ? r->s.err.c_str() : "null oracle";
}

int bromoc_ref_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int bromoc_ref_set_threads(int32_t n) {
#ifdef _OPENMP
  if (n < 1) return BROMOC_E_ARG;
  omp_set_num_threads(n);
#else
  (void)n;
#endif
  return BROMOC_OK;
}

int bromoc_ref_set_system(bromoc_ref *r, const bromoc_system *q) {
  if (!r || !q) return fail(r, "set_system: null");
  State &s = r->s;
  s.sys = *q;
  s.ikbt = 1.0 / q->kbt;
  s.kbtdt = q->dt * s.ikbt;  // simul1.f90:342
  // shell_simul.f90:914-919
  s.lx2p = q->cx + 0.5 * q->lx;
  s.ly2p = q->cy + 0.5 * q->ly;
  s.lz2p = q->cz + 0.5 * q->lz;
  s.lx2m = q->cx - 0.5 * q->lx;
  s.ly2m = q->cy - 0.5 * q->ly;
  s.lz2m = q->cz - 0.5 * q->lz;
  s.rsphe2 = q->rsphe * q->rsphe;
  if (q->shape == BROMOC_ECYL) {
    s.iecx = 2.0 / q->lx;
    s.iecy = 2.0 / q->ly;
  }
  s.have_sys = true;
  if (s.have_types) {
    for (int i = 1; i <= s.ntype; ++i) {
      s.fact1a[i] = s.diffusion[i] * s.kbtdt;
      s.fact2a[i] = std::sqrt(2.0 * q->dt * s.diffusion[i]);
    }
  }
  return BROMOC_OK;
}

int bromoc_ref_set_types(bromoc_ref *r, const bromoc_types *t) {
  if (!r || !t || !t->nwtype || !t->cg || !t->diffusion)
    return fail(r, "set_types: null");
  State &s = r->s;
  s.ntype = t->ntype;
  s.nold = t->nold;
  s.nttyp = t->nttyp;
  s.ndna = t->ndna;
  s.nion = s.nttyp - s.ndna;  // reasig.f90:310
  s.ndnaxnion = s.ndna * s.nion;
  s.nwtype = one_based(t->nwtype, t->ntype);
  s.cg = one_based(t->cg, t->ntype);
  s.diffusion = one_based(t->diffusion, t->ntype);
  s.fact1a.assign(s.ntype + 1, 0.0);
  s.fact2a.assign(s.ntype + 1, 0.0);
  s.warn.assign(s.nttyp + 1, 0);
  s.have_types = true;
  if (s.have_sys) bromoc_ref_set_system(r, &s.sys);
  return BROMOC_OK;
}

int bromoc_ref_set_pairs(bromoc_ref *r, const bromoc_pairs *p) {
  if (!r || !p) return fail(r, "set_pairs: null");
  State &s = r->s;
  const int n = p->ntc;
  s.ntc = n;
  s.qchr = one_based(p->qchr, n);
  s.qlj = one_based(p->qlj, n);
  s.qsrpmfi = one_based(p->qsrpmf, n);
  s.qefpot = one_based(p->qefpot, n);
  s.fct = one_based(p->fct, n);
  s.epp4 = one_based(p->epp4, n);
  s.sgp2 = one_based(p->sgp2, n);
  s.c0 = one_based(p->c0, n);
  s.c1 = one_based(p->c1, n);
  s.c2 = one_based(p->c2, n);
  s.c3 = one_based(p->c3, n);
  s.c4 = one_based(p->c4, n);
  s.rth = p->rth;
  s.srpx = p->srpx;
  s.srpk = p->srpk;
  s.srpy = p->srpy;
  s.cnt = p->cnt;
  s.ep.assign(p->ep ? p->ep : (const double *)nullptr,
              p->ep ? p->ep + 3 * (size_t)p->cnt : nullptr);
  s.sc.assign(3 * (size_t)n, 0.0);
  s.dm2.assign(2 * (size_t)n, 0.0);
  if (p->sc) std::memcpy(s.sc.data(), p->sc, 3 * sizeof(double) * n);
  if (p->dm2) std::memcpy(s.dm2.data(), p->dm2, 2 * sizeof(double) * n);
  s.dmi = one_based(p->dmi, n);
  s.nxi = one_based(p->nxi, n);
  s.res = p->res;
  s.ires = p->res > 0 ? 1.0 / p->res : 0.0;
  s.have_pairs = true;
  return BROMOC_OK;
}

int bromoc_ref_set_sites(bromoc_ref *r, const bromoc_sites *q) {
  if (!r || !q) return fail(r, "set_sites: null");
  State &s = r->s;
  s.nsites = q->nsites;
  s.nuc = bref::Nucl{};  // the term lists name sites of the previous set
  s.typtyp = one_based(q->typtyp, q->nsites);
  s.sitecharge = one_based(q->charge, q->nsites);
  s.stfree = one_based(q->stfree, q->nsites);
  s.site_phiv_map = one_based(q->phiv_map, q->nsites);
  return BROMOC_OK;
}

int bromoc_ref_set_nucleotides(bromoc_ref *r, const bromoc_nucleotides *q) {
  if (!r) return BROMOC_E_ARG;
  State &s = r->s;
  s.nuc = bref::Nucl{};
  if (!q) return BROMOC_OK;
  const int ns = s.nsites;
  bool bad = false;
  auto list = [&](int n, const int32_t *v, int per, std::vector<int> &out) {
    if (n < 0 || (n > 0 && !v)) bad = true;
    if (bad || n <= 0) return;
    out.assign(v, v + (size_t)n * per);
    for (int k : out)
      if (k < 1 || k > ns) bad = true;
  };
  auto vals = [&](int n, const double *v, std::vector<double> &out) {
    if (n > 0 && !v) bad = true;
    if (!bad && n > 0) out.assign(v, v + n);
  };
  bref::Nucl &n = s.nuc;
  list(q->nbond, q->sitebond, 2, n.bond);
  vals(q->nbond, q->distbond, n.distbond);
  list(q->nangle, q->siteangle, 3, n.angle);
  vals(q->nangle, q->valangle, n.valangle);
  list(q->ndihe, q->sitedihe, 4, n.dihe);
  vals(q->ndihe, q->valdihe, n.valdihe);
  list(q->nstack, q->sitestack, 2, n.stack);
  vals(q->nstack, q->sgstack, n.sgstack);
  list(q->nbp, q->sitebp, 2, n.bp);
  vals(q->nbp, q->sgbp, n.sgbp);
  if (q->nbp > 0 && !q->bpgc) bad = true;
  if (!bad && q->nbp > 0) n.bpgc.assign(q->bpgc, q->bpgc + q->nbp);
  list(q->nex, q->siteex, 2, n.ex);
  vals(q->nex, q->sgex, n.sgex);
  list(q->nqq, q->siteqq, 2, n.qq);
  list(q->nsolv, q->siteslv, 2, n.slv);
  list(q->afn, q->sn, 1, n.sn);
  if (q->afn > 0 && !q->af) bad = true;
  if (!bad && q->afn > 0) n.af.assign(q->af, q->af + 3 * (size_t)q->afn);
  if (q->ctn < 0 || (q->ctn > 0 && (!q->csn || !q->kx || !q->ky || !q->kz || !q->contrx ||
                                     !q->contry || !q->contrz)))
    bad = true;
  if (!bad && q->ctn > 0) {
    n.csn.assign(q->csn, q->csn + q->ctn);
    for (int k : n.csn)
      if (k < 0 || k > ns) bad = true;
    n.kx.assign(q->kx, q->kx + q->ctn);
    n.ky.assign(q->ky, q->ky + q->ctn);
    n.kz.assign(q->kz, q->kz + q->ctn);
    n.contrx.assign(q->contrx, q->contrx + q->ctn + 1);
    n.contry.assign(q->contry, q->contry + q->ctn + 1);
    n.contrz.assign(q->contrz, q->contrz + q->ctn + 1);
  }
  if (q->qunsplit && (q->nsites1st < 1 || q->nsites1st >= ns)) bad = true;
  if (q->qdeby && !(q->kappa > 0.0)) bad = true;
  if (bad || ns <= 0) {
    s.nuc = bref::Nucl{};
    return fail(r, "set_nucleotides: bad list, site number or count");
  }
  n.epsnuc = q->epsnuc;
  n.scalepairing = q->scalepairing;
  n.fctn = q->fctn;
  n.kappa = q->kappa;
  n.ikappa = q->qdeby ? 1.0 / q->kappa : 0.0;
  n.qdeby = q->qdeby;
  n.qsolv = q->qsolv != 0;
  n.epsolv = q->epsolv;
  n.qunsplit = q->qunsplit != 0;
  n.nsites1st = q->nsites1st;
  for (int a = 0; a < 3; ++a) {
    n.qnotr[a] = q->qnotr[a] != 0;
    n.notr[a] = q->notr[a];
  }
  n.on = true;
  return BROMOC_OK;
}

int bromoc_ref_set_mmij(bromoc_ref *r, const bromoc_mmij *q) {
  if (!r) return BROMOC_E_ARG;
  State &s = r->s;
  s.mm = bref::Mmij{};
  if (!q) return BROMOC_OK;
  bref::Mmij &m = s.mm;
  if (q->shape == BROMOC_BOX) {
    if (q->xnpol < 1 || q->ynpol < 1 || q->znpol < 1 || !q->lstpx || !q->lstpy || !q->lstpz ||
        !q->mmij || !(q->rbxmax - q->rbxmin > 0.0) || !(q->rbymax - q->rbymin > 0.0) ||
        !(q->rbzmax - q->rbzmin > 0.0))
      return fail(r, "set_mmij: RECTBOX orders, region or matrix");
    m.rect = true;
    m.xnpol = q->xnpol;
    m.ynpol = q->ynpol;
    m.znpol = q->znpol;
    m.ntpol = q->xnpol * q->ynpol * q->znpol;
    m.lstpx.assign(q->lstpx, q->lstpx + m.ntpol);
    m.lstpy.assign(q->lstpy, q->lstpy + m.ntpol);
    m.lstpz.assign(q->lstpz, q->lstpz + m.ntpol);
    for (int n = 0; n < m.ntpol; ++n)
      if (m.lstpx[n] < 0 || m.lstpx[n] >= m.xnpol || m.lstpy[n] < 0 || m.lstpy[n] >= m.ynpol ||
          m.lstpz[n] < 0 || m.lstpz[n] >= m.znpol) {
        s.mm = bref::Mmij{};
        return fail(r, "set_mmij: order out of range");
      }
    // shell_simul.f90:2792-2802
    m.xscal = 2.0 / (q->rbxmax - q->rbxmin);
    m.yscal = 2.0 / (q->rbymax - q->rbymin);
    m.zscal = 2.0 / (q->rbzmax - q->rbzmin);
    m.xmin = -1.0 / m.xscal;
    m.xmax = 1.0 / m.xscal;
    m.ymin = -1.0 / m.yscal;
    m.ymax = 1.0 / m.yscal;
    m.zmin = -1.0 / m.zscal;
    m.zmax = 1.0 / m.zscal;
    m.rfscal = q->rfscal;
  } else if (q->shape == BROMOC_SPHERE) {
    if (q->nmpol < 1 || q->nmpol > 25 || !(q->srdist > 0.0) || !q->mmij)
      return fail(r, "set_mmij: SPHERE nmpol, srdist or matrix");
    m.rect = false;
    m.nmpol = q->nmpol;
    m.ntpol = q->nmpol * q->nmpol;
    m.srdist = q->srdist;
  } else {
    return fail(r, "set_mmij: shape must be RECTBOX or SPHERE");
  }
  const int nt = m.ntpol;
  m.mmij.assign(q->mmij, q->mmij + (size_t)nt * nt);
  for (int i = 0; i < nt; ++i)  // readmmij.f90: mmij(ij) = mmij(ji) for i > j
    for (int j = 0; j < i; ++j) m.mmij[(size_t)i * nt + j] = m.mmij[(size_t)j * nt + i];
  bref::mmij_basis(m);
  m.on = true;
  return BROMOC_OK;
}

int bromoc_ref_set_phix(bromoc_ref *r, const bromoc_grid *g, const float *phix) {
  if (!r || !g || !phix) return fail(r, "set_phix: null");
  State &s = r->s;
  s.g1.set(*g);
  s.phix.assign(phix, phix + (size_t)g->nclx * g->ncly * g->nclz);
  s.qphix = true;
  return BROMOC_OK;
}

int bromoc_ref_set_phiv(bromoc_ref *r, const bromoc_grid *g, const int8_t *phiv,
                        const bromoc_phiv_opts *o) {
  if (!r || !g || !phiv || !o) return fail(r, "set_phiv: null");
  State &s = r->s;
  s.g2.set(*g);
  s.phiv_nmaps = o->nmaps;
  s.phiv.assign(phiv, phiv + (size_t)o->nmaps * g->nclx * g->ncly * g->nclz);
  s.qtrln = o->trilinear != 0;
  s.qnmcden = o->nmcden != 0;
  s.svdw = o->svdw;
  s.vzmin = o->vzmin;
  s.vzmax = o->vzmax;
  s.thold8 = o->thold8;
  s.thold27 = o->thold27;
  s.phiv_map_of_type = one_based(o->map_of_type, s.ntype);
  s.qsvdw = o->scal != nullptr;
  s.scal = one_based(o->scal, s.nttyp);
  s.qphiv = true;
  return BROMOC_OK;
}

int bromoc_ref_set_rfpar(bromoc_ref *r, const bromoc_grid *g, int32_t nmaps,
                         const float *gsrfen, const float *greff, double reffac,
                         const int32_t *map_of_type) {
  if (!r || !g || !gsrfen || !greff) return fail(r, "set_rfpar: null");
  State &s = r->s;
  s.g3.set(*g);
  size_t n = (size_t)nmaps * g->nclx * g->ncly * g->nclz;
  s.gsrfen.assign(gsrfen, gsrfen + n);
  s.greff.assign(greff, greff + n);
  s.sqrfac = std::sqrt(reffac);  // shell_simul.f90:2860
  s.qrfpsin = map_of_type == nullptr;
  s.rfpar_map_of_type = one_based(map_of_type, s.ntype);
  s.qrfpar = true;
  return BROMOC_OK;
}

int bromoc_ref_set_membrane(bromoc_ref *r, const bromoc_membrane *m) {
  if (!r || !m) return fail(r, "set_membrane: null");
  State &s = r->s;
  const int n = s.nttyp;
  s.qpore = m->qpore != 0;
  s.voltage = m->voltage;
  s.afact = m->afact;
  s.ikappa = m->ikappa;
  s.ceps = m->ceps;
  s.zmemb1 = m->zmemb1;
  s.zmemb2 = m->zmemb2;
  s.ampl1 = one_based(m->ampl1, n);
  s.ampl2 = one_based(m->ampl2, n);
  s.rcylinder = one_based(m->rcylinder, n);
  s.p1a.assign(n + 1, 1.0);
  s.p1b.assign(n + 1, 1.0);
  s.p2a.assign(n + 1, 1.0);
  s.p2b.assign(n + 1, 1.0);
  for (int i = 1; i <= n; ++i) {
    s.p1a[i] = m->p1[2 * (i - 1)];
    s.p1b[i] = m->p1[2 * (i - 1) + 1];
    s.p2a[i] = m->p2[2 * (i - 1)];
    s.p2b[i] = m->p2[2 * (i - 1) + 1];
  }
  s.qmemb = true;
  return BROMOC_OK;
}

int bromoc_ref_set_diffusion(bromoc_ref *r, const bromoc_diffusion *d) {
  if (!r || !d) return fail(r, "set_diffusion: null");
  State &s = r->s;
  s.dif = *d;
  s.ampl3 = one_based(d->ampl3, s.ntype);
  s.p3 = one_based(d->p3, s.ntype);
  s.xs = one_based(d->xs, d->nspline);
  s.ys = one_based(d->ys, d->nspline);
  s.sb = one_based(d->b, d->nspline);
  s.scc = one_based(d->c, d->nspline);
  s.sd = one_based(d->d, d->nspline);
  s.have_dif = true;
  return BROMOC_OK;
}

int bromoc_ref_set_periodic(bromoc_ref *r, int32_t on, double rcut) {
  if (!r) return BROMOC_E_ARG;
  State &s = r->s;
  if (on && (!s.have_sys || s.sys.shape != BROMOC_BOX))
    return fail(r, "set_periodic: needs set_system with a box");
  if (on && !(rcut > 0.0)) return fail(r, "set_periodic: rcut must be > 0");
  s.periodic = on != 0;
  s.rcut2 = on ? rcut * rcut : 0.0;
  return BROMOC_OK;
}

int bromoc_ref_set_countions(bromoc_ref *r, int32_t cntpts, const double *zcont) {
  if (!r || cntpts < 0 || (cntpts > 0 && !zcont)) return fail(r, "set_countions");
  State &s = r->s;
  s.cntpts = cntpts;
  s.zcont = one_based(zcont, cntpts);
  size_t n = (size_t)(s.ntype - s.nold) * cntpts;
  s.nforward.assign(n, 0);
  s.nbackward.assign(n, 0);
  return BROMOC_OK;
}

int bromoc_ref_set_buffers(bromoc_ref *r, const bromoc_buffers *b) {
  if (!r || !b) return fail(r, "set_buffers: null");
  State &s = r->s;
  const int n = b->nbuffer;
  s.nbuffer = n;
  s.ibfftyp = one_based(b->ibfftyp, n);
  s.avnum = one_based(b->avnum, n);
  s.mu = one_based(b->mu, n);
  s.kb = one_based(b->kb, n);
  s.lzmin = one_based(b->lzmin, n);
  s.lzmax = one_based(b->lzmax, n);
  s.rmin = one_based(b->rmin, n);
  s.rmax = one_based(b->rmax, n);
  s.qbufferbias = one_based(b->qbufferbias, n);
  s.nat = one_based(b->nat, n);
  s.ntotat = one_based(b->ntotat, n);
  s.ninsert.assign(n + 1, 0);
  s.nremove.assign(n + 1, 0);
  s.prob.assign((size_t)n * (s.capacity + 1), 0);
  return BROMOC_OK;
}

int bromoc_ref_set_particles(bromoc_ref *r, int32_t ntot, int32_t nsites,
                             int32_t nfix, const double *x, const double *y,
                             const double *z, const int32_t *typei,
                             const int32_t *ibuffer) {
  if (!r || !x || !y || !z || !typei) return fail(r, "set_particles: null");
  State &s = r->s;
  if (ntot > s.capacity) return fail(r, "ntot exceeds capacity", BROMOC_E_CAPACITY);
  if (nsites != s.nsites) return fail(r, "nsites differs from set_sites", BROMOC_E_STATE);
  s.ntot = ntot;
  s.nfix = nfix;
  for (int i = 0; i < ntot; ++i) {
    s.x[i + 1] = x[i];
    s.y[i + 1] = y[i];
    s.z[i + 1] = z[i];
    s.typei[i + 1] = typei[i];
    s.ibuffer[i + 1] = ibuffer ? ibuffer[i] : 0;
  }
  return BROMOC_OK;
}

int bromoc_ref_get_particles(bromoc_ref *r, int32_t *ntot, double *x, double *y,
                             double *z, int32_t *typei, int32_t *ibuffer) {
  if (!r) return BROMOC_E_ARG;
  State &s = r->s;
  if (ntot) *ntot = s.ntot;
  for (int i = 0; i < s.ntot; ++i) {
    if (x) x[i] = s.x[i + 1];
    if (y) y[i] = s.y[i + 1];
    if (z) z[i] = s.z[i + 1];
    if (typei) typei[i] = s.typei[i + 1];
    if (ibuffer) ibuffer[i] = s.ibuffer[i + 1];
  }
  return BROMOC_OK;
}

static void terms_out(const State &s, double *e) {
  if (!e) return;
  e[BROMOC_ENER] = s.ener;
  e[BROMOC_EELEC] = s.eelec;
  e[BROMOC_EVDW] = s.evdw;
  e[BROMOC_ESRPMF] = s.esrpmf;
  e[BROMOC_EEFPOT] = s.eefpot;
  e[BROMOC_EQQMX] = s.eqqmx;
  e[BROMOC_EVDWMX] = s.evdwmx;
  e[BROMOC_ESRPMFMX] = s.esrpmfmx;
  e[BROMOC_EEFPOTMX] = s.eefpotmx;
  e[BROMOC_EMEMB] = s.ememb;
  e[BROMOC_EGSBPA] = s.egsbpa;
  e[BROMOC_EGSBPB] = s.egsbpb;
  e[BROMOC_EVDWGD] = s.evdwgd;
  e[BROMOC_ERFPAR] = s.erfpar;
  e[BROMOC_EBOND] = s.ebond;
  e[BROMOC_EANG] = s.eang;
  e[BROMOC_EDIHE] = s.edihe;
  e[BROMOC_ESTACK] = s.estack;
  e[BROMOC_EBP] = s.ebp;
  e[BROMOC_EEX] = s.eex;
  e[BROMOC_EQQ] = s.eqq;
  e[BROMOC_ESOLV] = s.esolv;
  e[BROMOC_ECON] = s.econ;
}

static bool ready(bromoc_ref *r) {
  State &s = r->s;
  if (!s.have_sys || !s.have_types || !s.have_pairs) {
    s.err = "set_system, set_types and set_pairs are required";
    return false;
  }
  if (s.periodic && (s.nsites > 0 || s.qrfpar)) {  // the extension mode's scope
    s.err = "periodic mode: ions only, without RFPAR";
    return false;
  }
  return true;
}

int bromoc_ref_energy(bromoc_ref *r, uint32_t terms, int32_t qforces,
                      double *fx, double *fy, double *fz, double *eterms,
                      int32_t *warn) {
  if (!r) return BROMOC_E_ARG;
  if (!ready(r)) return BROMOC_E_STATE;
  State &s = r->s;
  std::fill(s.warn.begin(), s.warn.end(), 0);
  bref::energy(s, terms, qforces != 0);
  terms_out(s, eterms);
  if (qforces)
    for (int i = 0; i < s.ntot; ++i) {
      if (fx) fx[i] = s.fx[i + 1];
      if (fy) fy[i] = s.fy[i + 1];
      if (fz) fz[i] = s.fz[i + 1];
    }
  if (warn)
    for (int i = 0; i < s.nttyp; ++i) warn[i] = s.warn[i + 1];
  return BROMOC_OK;
}

int bromoc_ref_interact(bromoc_ref *r, uint32_t terms, double xj, double yj,
                        double zj, int32_t jtype, int32_t j, double *dener) {
  if (!r || !dener) return BROMOC_E_ARG;
  if (!ready(r)) return BROMOC_E_STATE;
  State &s = r->s;
  if (j < 1 || j > s.ntot + 1) return fail(r, "interact: j out of range");
  if (j == s.ntot + 1 && s.ntot + 1 > s.capacity)
    return fail(r, "interact: no room for the trial slot", BROMOC_E_CAPACITY);
  bref::interact(s, terms, *dener, xj, yj, zj, jtype, j, true);
  return BROMOC_OK;
}

int bromoc_ref_dynamics(bromoc_ref *r, int32_t variant, uint64_t seed,
                        uint64_t step) {
  if (!r) return BROMOC_E_ARG;
  if (!ready(r)) return BROMOC_E_STATE;
  bref::dynamics(r->s, variant, seed, step);
  return BROMOC_OK;
}

int bromoc_ref_bd_steps(bromoc_ref *r, uint32_t terms, int32_t variant,
                        int32_t nsteps, uint64_t seed, uint64_t step0,
                        double *eterms) {
  if (!r) return BROMOC_E_ARG;
  if (!ready(r)) return BROMOC_E_STATE;
  for (int k = 0; k < nsteps; ++k) {
    bref::energy(r->s, terms, true);
    bref::dynamics(r->s, variant, seed, step0 + k);
  }
  terms_out(r->s, eterms);
  return BROMOC_OK;
}

int bromoc_ref_grand(bromoc_ref *r, uint32_t terms, int32_t ngcmc, uint64_t seed,
                     uint64_t cycle, double *dener_sum) {
  if (!r) return BROMOC_E_ARG;
  if (!ready(r)) return BROMOC_E_STATE;
  if (cycle < 1) return fail(r, "grand: cycle is 1-based");
  double d = 0.0;
  r->s.err.clear();
  bref::grand(r->s, terms, ngcmc, seed, cycle, d);
  if (dener_sum) *dener_sum = d;
  return r->s.err.empty() ? BROMOC_OK : BROMOC_E_CAPACITY;
}

int bromoc_ref_metropolis(bromoc_ref *r, uint32_t terms, int32_t nmcm, double mcmax,
                          uint64_t seed, uint64_t cycle, int32_t *naccept,
                          double *dener_sum) {
  if (!r || nmcm < 0 || !(mcmax > 0.0)) return BROMOC_E_ARG;
  if (!ready(r)) return BROMOC_E_STATE;
  if (r->s.nfix > 0) return fail(r, "metropolis: systems with fixed ions are not supported",
                                 BROMOC_E_STATE);
  if (r->s.ntot - r->s.nsites < 1) return fail(r, "metropolis: no mobile ion", BROMOC_E_STATE);
  double d = 0.0;
  int na = 0;
  bref::metropolis(r->s, terms, nmcm, mcmax, seed, cycle, d, na);
  if (naccept) *naccept = na;
  if (dener_sum) *dener_sum = d;
  return BROMOC_OK;
}

int bromoc_ref_count(bromoc_ref *r) {
  if (!r) return BROMOC_E_ARG;
  State &s = r->s;
  if (s.nbuffer < 1) return BROMOC_OK;
  if (!bref::count(s)) return fail(r, "count: particles outside main system", BROMOC_E_DEVICE);
  return BROMOC_OK;
}

int bromoc_ref_get_ntotat(bromoc_ref *r, int32_t *ntotat) {
  if (!r || !ntotat) return BROMOC_E_ARG;
  for (int i = 0; i < r->s.nbuffer; ++i) ntotat[i] = r->s.ntotat[i + 1];
  return BROMOC_OK;
}

int bromoc_ref_get_buffers(bromoc_ref *r, int32_t *nat, int32_t *ninsert,
                           int32_t *nremove, int32_t *prob) {
  if (!r) return BROMOC_E_ARG;
  State &s = r->s;
  for (int i = 0; i < s.nbuffer; ++i) {
    if (nat) nat[i] = s.nat[i + 1];
    if (ninsert) ninsert[i] = s.ninsert[i + 1];
    if (nremove) nremove[i] = s.nremove[i + 1];
  }
  if (prob) std::memcpy(prob, s.prob.data(), s.prob.size() * sizeof(int32_t));
  return BROMOC_OK;
}

int bromoc_ref_get_countions(bromoc_ref *r, int32_t *nf, int32_t *nb) {
  if (!r) return BROMOC_E_ARG;
  State &s = r->s;
  if (nf) std::memcpy(nf, s.nforward.data(), s.nforward.size() * sizeof(int32_t));
  if (nb) std::memcpy(nb, s.nbackward.data(), s.nbackward.size() * sizeof(int32_t));
  return BROMOC_OK;
}

int bromoc_ref_get_dids(bromoc_ref *r, double *dids) {
  if (!r || !dids) return BROMOC_E_ARG;
  std::memcpy(dids, r->s.dids.data(), 5 * sizeof(double) * r->s.ntot);
  return BROMOC_OK;
}

int bromoc_ref_efpot_from_knots(int32_t n, const double *xx, const double *yy,
                                double fct, int32_t qchr, double *ep,
                                double *sc3, double *dm2o, double *dmio) {
  if (n < 3 || !xx || !yy || !ep || !sc3 || !dm2o || !dmio) return BROMOC_E_ARG;
  if (xx[0] == 0.0 || xx[n - 1] == 0.0) return BROMOC_E_ARG;  // splinepot:32
  bref::splinepot(n, xx, yy, fct, qchr != 0, ep, sc3, dm2o, dmio);
  return BROMOC_OK;
}

void bromoc_ref_philox(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]) {
  bref::philox4x32_10(ctr, key, out);
}
double bromoc_ref_bd_gauss(uint64_t seed, uint64_t step, uint32_t slot,
                           int32_t comp) {
  return bref::bd_gauss(seed, step, slot, comp);
}
double bromoc_ref_gcmc_uniform(uint64_t seed, uint64_t cycle, uint32_t attempt,
                               uint32_t draw) {
  return bref::gcmc_uniform(seed, cycle, attempt, draw);
}
void bromoc_ref_squarespline(int32_t n, const double *x, const double *y,
                             double *p, double d1, double d2, double dd2) {
  bref::squarespline(n, x, y, p, d1, d2, dd2);
}

}  // extern "C"
