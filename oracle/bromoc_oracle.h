/* ORACLE -- test infrastructure only.  C API of the CPU FP64 restatement of
 * the cg-gcmc-bd hot path; same arguments as the bromoc_gpu_* entry points
 * of include/bromoc_gpu.h so that tests feed both with identical inputs.
 * Parity with the reference's own outputs is unpinned (see ref_state.h). */
#ifndef BROMOC_ORACLE_H
#define BROMOC_ORACLE_H
#include "../include/bromoc_gpu.h"
#ifdef __cplusplus
extern "C" {
#endif
typedef struct bromoc_ref bromoc_ref;
int bromoc_ref_create(int32_t capacity, bromoc_ref **out);
int bromoc_ref_destroy(bromoc_ref *r);
const char *bromoc_ref_last_error(const bromoc_ref *r);
int bromoc_ref_threads(void);
/* OpenMP threads of the timed build (no effect on the sequential one). */
int bromoc_ref_set_threads(int32_t n);
int bromoc_ref_metropolis(bromoc_ref *r, uint32_t terms, int32_t nmcm, double mcmax,
                          uint64_t seed, uint64_t cycle, int32_t *naccept,
                          double *dener_sum);
int bromoc_ref_set_system(bromoc_ref *r, const bromoc_system *sys);
int bromoc_ref_set_types(bromoc_ref *r, const bromoc_types *t);
int bromoc_ref_set_pairs(bromoc_ref *r, const bromoc_pairs *p);
int bromoc_ref_set_sites(bromoc_ref *r, const bromoc_sites *s);
int bromoc_ref_set_nucleotides(bromoc_ref *r, const bromoc_nucleotides *n);
int bromoc_ref_set_mmij(bromoc_ref *r, const bromoc_mmij *m);
int bromoc_ref_set_phix(bromoc_ref *r, const bromoc_grid *g, const float *phix);
int bromoc_ref_set_phiv(bromoc_ref *r, const bromoc_grid *g,
                        const int8_t *phiv, const bromoc_phiv_opts *o);
int bromoc_ref_set_rfpar(bromoc_ref *r, const bromoc_grid *g, int32_t nmaps,
                         const float *gsrfen, const float *greff,
                         double reffac, const int32_t *map_of_type);
int bromoc_ref_set_membrane(bromoc_ref *r, const bromoc_membrane *m);
int bromoc_ref_set_diffusion(bromoc_ref *r, const bromoc_diffusion *d);
int bromoc_ref_set_periodic(bromoc_ref *r, int32_t on, double rcut);
int bromoc_ref_set_countions(bromoc_ref *r, int32_t cntpts,
                             const double *zcont);
int bromoc_ref_set_buffers(bromoc_ref *r, const bromoc_buffers *b);
int bromoc_ref_set_particles(bromoc_ref *r, int32_t ntot, int32_t nsites,
                             int32_t nfix, const double *x, const double *y,
                             const double *z, const int32_t *typei,
                             const int32_t *ibuffer);
int bromoc_ref_get_particles(bromoc_ref *r, int32_t *ntot, double *x,
                             double *y, double *z, int32_t *typei,
                             int32_t *ibuffer);
int bromoc_ref_energy(bromoc_ref *r, uint32_t terms, int32_t qforces,
                      double *fx, double *fy, double *fz, double *eterms,
                      int32_t *warn);
int bromoc_ref_interact(bromoc_ref *r, uint32_t terms, double xj, double yj,
                        double zj, int32_t jtype, int32_t j, double *dener);
int bromoc_ref_dynamics(bromoc_ref *r, int32_t variant, uint64_t seed,
                        uint64_t step);
int bromoc_ref_bd_steps(bromoc_ref *r, uint32_t terms, int32_t variant,
                        int32_t nsteps, uint64_t seed, uint64_t step0,
                        double *eterms);
int bromoc_ref_grand(bromoc_ref *r, uint32_t terms, int32_t ngcmc,
                     uint64_t seed, uint64_t cycle, double *dener_sum);
/* count.f90 (buffer membership, nat, ntotat) */
int bromoc_ref_count(bromoc_ref *r);
int bromoc_ref_get_ntotat(bromoc_ref *r, int32_t *ntotat);
int bromoc_ref_get_buffers(bromoc_ref *r, int32_t *nat, int32_t *ninsert,
                           int32_t *nremove, int32_t *prob);
int bromoc_ref_get_countions(bromoc_ref *r, int32_t *nforward,
                             int32_t *nbackward);
int bromoc_ref_get_dids(bromoc_ref *r, double *dids);
int bromoc_ref_efpot_from_knots(int32_t n, const double *xx, const double *yy,
                                double fct, int32_t qchr, double *ep,
                                double *sc3, double *dm2o, double *dmio);
/* building blocks exposed for unit tests */
void bromoc_ref_philox(const uint32_t ctr[4], const uint32_t key[2],
                       uint32_t out[4]);
double bromoc_ref_bd_gauss(uint64_t seed, uint64_t step, uint32_t slot,
                           int32_t comp);
double bromoc_ref_gcmc_uniform(uint64_t seed, uint64_t cycle,
                               uint32_t attempt, uint32_t draw);
void bromoc_ref_squarespline(int32_t n, const double *x, const double *y,
                             double *p, double d1, double d2, double dd2);
#ifdef __cplusplus
}
#endif
#endif
