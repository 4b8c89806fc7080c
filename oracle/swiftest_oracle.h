/*
 * swiftest_oracle.h -- CPU FP64 restatement of Swiftest's integrator hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker for the CUDA path in
 * swiftest_gb300/; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it.  The product never links or calls it.
 *
 * Parity status: the reference is Modern Fortran and cannot be compiled in the
 * build container (no Fortran compiler), and the reference's own test suite
 * holds no kernel-level golden vectors.  Parity of this restatement is pinned
 * by known-answer tests instead (analytic two-body Kepler propagation,
 * closed-form accelerations, hand-built encounter geometries, Newton's third
 * law, the reference's conservation-slope thresholds), see tests/.
 *
 * Conventions (mirroring the reference):
 *   - positions/velocities are Fortran (3,n) arrays: xyz of one body contiguous
 *   - body indices in encounter lists are 1-based int32
 *   - logical masks are int32 (0/1), like gfortran's 4-byte default logical
 *   - all arithmetic is IEEE binary64 with FP contraction disabled
 *     (-ffp-contract=off), evaluated in the reference's operation order.
 */
#ifndef SWIFTEST_ORACLE_H
#define SWIFTEST_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- kick: src/swiftest/swiftest_kick.f90 ---------------------------- */
void orc_kick_getacch_int_all_tri_pl(int32_t npl, int32_t nplm, const double *r, const double *Gmass,
                                     const double *radius /* NULL => norad */, double *acc);
void orc_kick_getacch_int_all_flat_pl(int32_t npl, int64_t nplpl, const int32_t *k_plpl, const double *r,
                                      const double *Gmass, const double *radius /* NULL => norad */,
                                      double *acc);
void orc_kick_getacch_int_all_tp(int32_t ntp, int32_t npl, const double *rtp, const double *rpl,
                                 const double *GMpl, const int32_t *lmask, double *acc);
int64_t orc_util_flatten_eucl_plpl(int32_t npl, int32_t nplm, int32_t *k_plpl /* NULL => count only */);

/* ---- drift: src/swiftest/swiftest_drift.f90 --------------------------- */
/* swiftest_orbel_el2xv_vec / _xv2el_vec: el[k*n+i] = (a, e, inc, capom, omega, capm)_k of body i;
 * out[k*n+i] = (a, e, inc, capom, omega, capm, varpi, lam, f, cape, capf)_k */
void orc_el2xv(int32_t n, const double *mu, const double *el, double *rh, double *vh);
void orc_xv2el(int32_t n, const double *mu, const double *rh, const double *vh, double *out);
void orc_drift_all(const double *mu, double *x, double *v, int32_t n, int32_t lgr, double inv_c2, double dt,
                   const int32_t *lmask, int32_t *iflag);
void orc_drift_one(double mu, double *rx, double *ry, double *rz, double *vx, double *vy, double *vz, double dt,
                   int32_t *iflag);
/* instrumented variant: returns number of Stumpff evaluations (FP64 work proxy) */
int64_t orc_drift_all_count(const double *mu, double *x, double *v, int32_t n, double dt, const int32_t *lmask,
                            int32_t *iflag);

/* ---- encounter: src/encounter/encounter_check.f90 ---------------------- */
#define ORC_ENC_TRIANGULAR 0
#define ORC_ENC_SORTSWEEP 1
void orc_encounter_check_one(double xr, double yr, double zr, double vxr, double vyr, double vzr, double renc,
                             double dt, int32_t *lencounter, int32_t *lvdotr);
/* Caller-capacity protocol: returns 0 on success, -3 if cap < *nenc (then
 * *nenc holds the required size and nothing beyond cap was written). */
int orc_encounter_check_all_plpl(int mode, int32_t npl, const double *r, const double *v, const double *renc,
                                 double dt, int64_t cap, int64_t *nenc, int32_t *index1, int32_t *index2,
                                 int32_t *lvdotr);
int orc_encounter_check_all_plplm(int mode, int32_t nplm, int32_t nplt, const double *rplm, const double *vplm,
                                  const double *rplt, const double *vplt, const double *rencm,
                                  const double *renct, double dt, int64_t cap, int64_t *nenc, int32_t *index1,
                                  int32_t *index2, int32_t *lvdotr);
int orc_encounter_check_all_pltp(int mode, int32_t npl, int32_t ntp, const double *rpl, const double *vpl,
                                 const double *rtp, const double *vtp, const double *renc, double dt,
                                 int64_t cap, int64_t *nenc, int32_t *index1, int32_t *index2, int32_t *lvdotr);

/* ---- nbody system + step loops (whm / helio / symba) ------------------- */
#define ORC_WHM 0
#define ORC_HELIO 1
#define ORC_SYMBA 2
typedef struct orc_system orc_system;
orc_system *orc_system_create(int integrator, int32_t npl, int32_t ntp);
void orc_system_destroy(orc_system *s);
/* central body: GM, radius */
void orc_system_set_cb(orc_system *s, double GMcb, double Rcb);
/* pl arrays: rh(3n), vh(3n), Gmass(n), radius(n), rhill(n); pl must be sorted by Gmass descending for helio/symba */
void orc_system_set_pl(orc_system *s, const double *rh, const double *vh, const double *Gmass, const double *radius,
                       const double *rhill);
void orc_system_set_tp(orc_system *s, const double *rh, const double *vh);
/* params: loop_mode 0 tri / 1 flat; encounter modes; rhscale; lclose; GMTINY (<=0 => off) */
void orc_system_set_param(orc_system *s, double dt, int loop_mode, int enc_plpl, int enc_pltp, double rhscale,
                          int lclose, double gmtiny);
int orc_system_initialize(orc_system *s); /* vh2vb, set_mu, eta (whm), flatten */
int orc_system_step(orc_system *s, int32_t nsteps);
void orc_system_get_pl(const orc_system *s, double *rh, double *vh, int32_t *status);
void orc_system_get_tp(const orc_system *s, double *rh, double *vh, int32_t *status);
int32_t orc_system_npl(const orc_system *s);
/* energy: te (total), L(3), ke_orbit, pe ; uses the reference's formulas */
void orc_system_energy(orc_system *s, double *out /* te, ke, pe, be, Lx, Ly, Lz, GMtot, te_helio */);
/* step-level counters: [n_steps_with_encounters, max_recursion_level, total_plpl_enc, total_pltp_enc, ncollisions,
 * recursion sub-steps] */
void orc_system_stats(const orc_system *s, int64_t *out);
/* out[4]: E_collisions, L_escape (x, y, z) booked by the collision resolution (G*m units) */
void orc_system_collision_terms(const orc_system *s, double *out);
/* last level-0 encounter lists */
int64_t orc_system_plpl_list(const orc_system *s, int64_t cap, int32_t *i1, int32_t *i2);
int64_t orc_system_pltp_list(const orc_system *s, int64_t cap, int32_t *i1, int32_t *i2);

#ifdef __cplusplus
}
#endif
#endif
