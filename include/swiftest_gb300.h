/*
 * swiftest_gb300.h -- C ABI of the GB300 (sm_103a) implementation of Swiftest's
 * integrator hot path: pair-gravity kick, Danby Kepler drift, close-encounter
 * checks, and the WHM / HELIO / SyMBA step loops that call them.
 *
 * Every entry point returns an int status (SWG_OK == 0, negative on error),
 * never aborts, never throws across the ABI.  Arrays follow the reference's
 * Fortran layout: positions and velocities are (3,n) column-major doubles
 * (x, y, z of one body contiguous); encounter indices are 1-based int32;
 * logical masks are int32 0/1 (gfortran's 4-byte default logical).
 *
 * Pointer arguments live in the memory space named by the `mem` argument:
 * SWG_MEM_HOST (copied to and from the GPU inside the call, which then
 * synchronizes) or SWG_MEM_DEVICE (device pointers; the call is ordered on
 * the context's stream and only synchronizes where a count must be returned).
 */
#ifndef SWIFTEST_GB300_H
#define SWIFTEST_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define SWG_OK 0
#define SWG_ERR_ARG (-1)       /* invalid argument */
#define SWG_ERR_CUDA (-2)      /* CUDA runtime error (message in swg_last_error) */
#define SWG_ERR_CAPACITY (-3)  /* output list too small; *nenc holds the required size */
#define SWG_ERR_NOMEM (-4)     /* device allocation failed */
#define SWG_ERR_DRIFT (-5)     /* Danby drift failed for a massive body in WHM (reference aborts) */
#define SWG_ERR_RECURSION (-6) /* SyMBA recursion step fell below machine epsilon */
#define SWG_ERR_STATE (-7)     /* call out of order (e.g. step before initialize) */

#define SWG_MEM_HOST 0
#define SWG_MEM_DEVICE 1

/* arithmetic of the pair kick */
#define SWG_FP64 0  /* FP64, reference operation order: bit-identical to the serial reference loop */
#define SWG_MIXED 1 /* FP64 positions split into float hi/lo, FP32 r^-3, float-float partial sums, FP64 total */

/* encounter-check modes (reference: param%lencounter_sas_plpl / _pltp) */
#define SWG_ENC_TRIANGULAR 0
#define SWG_ENC_SORTSWEEP 1

typedef struct swg_ctx swg_ctx;

/* Context: one per host thread; owns a CUDA stream and a grow-only device arena. */
int swg_create(swg_ctx **ctx, int device);
int swg_destroy(swg_ctx *ctx);
int swg_synchronize(swg_ctx *ctx);
const char *swg_last_error(const swg_ctx *ctx);
/* number of kernels this context has launched since creation */
int64_t swg_launch_count(const swg_ctx *ctx);

/* ---- pair-gravity kick ------------------------------------------------------
 * Replaces swiftest_kick_getacch_int_all_tri_rad_pl / _tri_norad_pl
 * (src/swiftest/swiftest_kick.f90:165-371; interface swiftest_module.f90:940-991).
 * acc is inout and accumulates like the reference.  radius == NULL selects the
 * norad variant.  nplm < npl selects the GMTINY (semi-interacting) loop shape. */
int swg_kick_getacch_int_all_tri_pl(swg_ctx *ctx, int32_t npl, int32_t nplm, const double *r, const double *Gmass,
                                    const double *radius, double *acc, int precision, int mem);

/* Replaces swiftest_kick_getacch_int_all_flat_rad_pl / _flat_norad_pl
 * (swiftest_kick.f90:69-162).  k_plpl is the (2,nplpl) 1-based pair list; pass
 * NULL for the canonical list built by swiftest_util_flatten_eucl_plpl
 * (swiftest_util.f90:1090-1131) restricted to rows i <= nplm, which the GPU
 * derives from tile coordinates instead of reading. */
int swg_kick_getacch_int_all_flat_pl(swg_ctx *ctx, int32_t npl, int32_t nplm, int64_t nplpl, const int32_t *k_plpl,
                                     const double *r, const double *Gmass, const double *radius, double *acc,
                                     int precision, int mem);

/* The mixed-precision pl-pl kick of swg_kick_getacch_int_all_tri_pl (SWG_MIXED) for callers
 * that cannot allocate device memory while they run: an application that owns every
 * device allocation in a fixed pool sized at start-up (a cudaMalloc mid-run could fail
 * or fragment that pool), or host code that keeps other streams busy and cannot let a
 * cudaMalloc/cudaFree synchronize the device.  It has no counterpart in the reference.  It calls no
 * cudaMalloc or cudaFree, takes device pointers and a cudaStream_t, and accumulates into
 * acc like the regular entry point.  It runs the regular entry point's broadcast kernel
 * on the same grid, so its results are the same bits wherever that entry point takes the
 * broadcast kernel (nplm < npl, or npl below about 12,000 on GB300); above that the regular
 * entry point switches to its symmetric kernel and the two agree within the mixed-kick
 * tolerance (per-body relative error 2e-5), not bit for bit.  Its scratch is one fixed
 * 16 MiB device array per GPU, held until exit and shared by all calls: it keeps the last
 * call's contents, the counters are cleared at the start of each call, and calls that
 * overlap on the GPU race.  npl above SWG_NOALLOC_MAX_NPL is rejected with SWG_ERR_ARG.
 * The first call on a device resolves the array's address: make it before any stream
 * capture (a first call on a capturing stream returns SWG_ERR_STATE). */
#define SWG_NOALLOC_MAX_NPL 1048576
int swg_kick_getacch_int_all_tri_pl_noalloc(int32_t npl, int32_t nplm, const double *r, const double *Gmass,
                                            const double *radius, double *acc, void *stream);

/* Replaces swiftest_kick_getacch_int_all_tp (swiftest_kick.f90:374-415). */
int swg_kick_getacch_int_all_tp(swg_ctx *ctx, int32_t ntp, int32_t npl, const double *rtp, const double *rpl,
                                const double *GMpl, const int32_t *lmask, double *acc, int precision, int mem);

/* ---- Danby drift ---------------------------------------------------------------
 * Replaces swiftest_drift_all (src/swiftest/swiftest_drift.f90:60-108; interface
 * swiftest_module.f90:513-522) including drift_one/_dan/_kepmd/_kepu*.
 * iflag gets the reference's per-body status (0 ok, 1 kepmd/Newton, 2 Laguerre). */
int swg_drift_all(swg_ctx *ctx, const double *mu, double *x, double *v, int32_t n, int32_t lgr, double inv_c2,
                  double dt, const int32_t *lmask, int32_t *iflag, int mem);

/* ---- encounter checks -----------------------------------------------------------
 * Replace encounter_check_all_plpl / _plplm / _pltp (src/encounter/encounter_check.f90:14-140).
 * Caller-capacity protocol (Fortran allocatable outputs cannot cross the ABI):
 * on return *nenc is the number of encounters; if it exceeds cap the call
 * returns SWG_ERR_CAPACITY and the caller retries with a larger buffer.
 * Output order is (index1, index2) ascending; lvdotr is int32 0/1. */
int swg_encounter_check_all_plpl(swg_ctx *ctx, int mode, int32_t npl, const double *r, const double *v,
                                 const double *renc, double dt, int64_t cap, int64_t *nenc, int32_t *index1,
                                 int32_t *index2, int32_t *lvdotr, int mem);
int swg_encounter_check_all_plplm(swg_ctx *ctx, int mode, int32_t nplm, int32_t nplt, const double *rplm,
                                  const double *vplm, const double *rplt, const double *vplt, const double *rencm,
                                  const double *renct, double dt, int64_t cap, int64_t *nenc, int32_t *index1,
                                  int32_t *index2, int32_t *lvdotr, int mem);
int swg_encounter_check_all_pltp(swg_ctx *ctx, int mode, int32_t npl, int32_t ntp, const double *rpl,
                                 const double *vpl, const double *rtp, const double *vtp, const double *renc,
                                 double dt, int64_t cap, int64_t *nenc, int32_t *index1, int32_t *index2,
                                 int32_t *lvdotr, int mem);

/* ---- sorting -------------------------------------------------------------------------
 * Replaces util_sort(arr, ind) (src/base/base_module.f90:1361-1472), the index quicksort the
 * sort-and-sweep check sorts its extents with: ind gets the 1-based permutation that orders
 * arr ascending.  Stable LSD radix sort on the GPU; equal values (-0.0 and +0.0 included)
 * keep their index order, where the reference's quicksort, seeded with the previous order,
 * leaves ties in an order that depends on history. */
int swg_util_sort_index(swg_ctx *ctx, int64_t n, const double *arr, int32_t *ind, int mem);

/* ---- device-resident n-body system and step loops ---------------------------------
 * Mirrors swiftest_nbody_system with whm_step_system (src/whm/whm_step.f90:14-104),
 * helio_step_system (src/helio/helio_step.f90:14-119) and symba_step_system
 * (src/symba/symba_step.f90:14-331).  State stays in HBM between steps. */
#define SWG_WHM 0
#define SWG_HELIO 1
#define SWG_SYMBA 2
typedef struct swg_system swg_system;
int swg_system_create(swg_ctx *ctx, int integrator, int32_t npl, int32_t ntp, swg_system **sys);
int swg_system_destroy(swg_system *sys);
int swg_system_set_cb(swg_system *sys, double GMcb, double Rcb);
/* host arrays; massive bodies sorted as the reference's initialize does
 * (HELIO/SyMBA: by mass descending; WHM: by heliocentric distance) */
int swg_system_set_pl(swg_system *sys, const double *rh, const double *vh, const double *Gmass, const double *radius,
                      const double *rhill);
int swg_system_set_tp(swg_system *sys, const double *rh, const double *vh);
/* loop_mode 0 triangular / 1 flat; encounter modes; rhscale (reference: 6.5);
 * lclose; gmtiny (<= 0 off); precision of the pair kick */
int swg_system_set_param(swg_system *sys, double dt, int loop_mode, int enc_plpl, int enc_pltp, double rhscale,
                         int lclose, double gmtiny, int precision);
int swg_system_initialize(swg_system *sys);
int swg_system_step(swg_system *sys, int32_t nsteps);
int swg_system_get_pl(swg_system *sys, double *rh, double *vh, int32_t *status);
int swg_system_get_tp(swg_system *sys, double *rh, double *vh, int32_t *status);
/* Current Gmass, radius and rhill of the massive bodies (a collision merge changes them; any
 * pointer may be NULL): what the reference's frame writer reads from pl%Gmass, pl%radius and
 * pl%rhill (swiftest_io_netcdf_write_frame_body, swiftest_io.f90:1837-1996). */
int swg_system_get_pl_masses(swg_system *sys, double *Gmass, double *radius, double *rhill);
/* out[9]: te, ke, pe, be, Lx, Ly, Lz, GMtot (swiftest_util.f90:1172-1401, whose central-body
 * potential uses the body's barycentric distance), then te_helio: the same total with the
 * central-body potential at the heliocentric distance. */
int swg_system_energy(swg_system *sys, double *out);
/* out[4]: the collision bookkeeping of swiftest_nbody_system (swiftest_module.f90:375-377):
 * E_collisions, the energy change of the collision resolutions (collision_resolve.f90:634-638),
 * and L_escape (x, y, z), the impactors' pre-collision orbital angular momentum
 * (collision_generate.f90:218-220), since initialize.  Masses enter as G*m, so both are G
 * times the reference's, like every value of swg_system_energy.  The reference's error
 * terms (swiftest_io.f90:153,181-183) follow: |dE/E| = |te - te0 - E_collisions| / |te0|,
 * |dL/L| = |L + L_escape - L0| / |L0|. */
int swg_system_collision_terms(swg_system *sys, double *out);
/* out[6]: steps with encounters, max recursion depth, sum plpl enc, sum pltp enc, collisions
 * resolved plus test particles removed by the close-approach discard scan, recursion
 * sub-steps executed */
int swg_system_stats(swg_system *sys, int64_t *out);
/* level-0 encounter lists of the last step */
int swg_system_plpl_list(swg_system *sys, int64_t cap, int64_t *n, int32_t *i1, int32_t *i2);
int swg_system_pltp_list(swg_system *sys, int64_t cap, int64_t *n, int32_t *i1, int32_t *i2);

/* Upload / download the integrator state (positions and heliocentric velocities of
 * massive bodies and test particles) of an initialized system without resetting its
 * step flags: the per-step exchange a host-side caller that owns the arrays performs.
 * NULL pointers are skipped.  get_state_async is ordered on the stream; call
 * swg_synchronize before reading the host arrays.
 * Like the reference's steps, a step after the first carries state of its own from the
 * step before (HELIO/SyMBA: the barycentric velocities pl%vb, tp%vb; WHM: the closing
 * accelerations), so an upload that changes the state reaches the next step only after
 * swg_system_reset_first_step, which sets the reference's lfirst flags (helio_step_pl,
 * whm_step_pl): the next step converts vh to vb and evaluates its opening accelerations
 * afresh, as the first step after swg_system_initialize does. */
int swg_system_set_state(swg_system *sys, const double *rh, const double *vh, const double *trh, const double *tvh);
int swg_system_get_state_async(swg_system *sys, double *rh, double *vh, double *trh, double *tvh);
int swg_system_reset_first_step(swg_system *sys);

/* ---- orbital elements <-> Cartesian state (swiftest_orbel_el2xv_vec / _xv2el_vec,
 * swiftest_orbel.f90:14-42, 876-910, with swiftest_orbel_el2xv :45-144 and swiftest_orbel_xv2el
 * :913-1072).  Body i uses mu[i] (GMcb + Gm for massive bodies, GMcb for test particles, as
 * set_mu does); angles in radians; rh, vh are (3, n).  xv2el also returns the longitude of
 * pericentre, mean longitude, true, eccentric and hyperbolic anomalies; any output pointer may
 * be NULL.  FP64; the transcendental functions are CUDA's (last-bit differences from libm). */
int swg_orbel_el2xv(swg_ctx *ctx, int32_t n, const double *mu, const double *a, const double *e, const double *inc,
                    const double *capom, const double *omega, const double *capm, double *rh, double *vh, int mem);
int swg_orbel_xv2el(swg_ctx *ctx, int32_t n, const double *mu, const double *rh, const double *vh, double *a,
                    double *e, double *inc, double *capom, double *omega, double *capm, double *varpi, double *lam,
                    double *f, double *cape, double *capf, int mem);

/* ---- batched ensembles of independent systems -------------------------------------
 * No single counterpart in the reference, which integrates one system per run: an
 * ensemble is many runs of whm_step_system / helio_step_system / symba_step_system
 * (whm_step.f90:14-104, helio_step.f90:14-119, symba_step.f90:14-331) advanced together,
 * each system taking exactly the steps it would take alone (bit-identical in SWG_FP64).
 * Systems are packed CSR-style: arrays of massive bodies are the concatenation of every
 * system's (3, npl[s]) block in system order (test particles likewise with ntp[s]), each
 * block ordered as the reference's initialize leaves it (HELIO/SyMBA: by mass, descending;
 * WHM: input order).  All systems share dt; GMTINY is not supported.  integrator: SWG_WHM,
 * SWG_HELIO or SWG_SYMBA (level-0 checks TRIANGULAR unless swg_ensemble_set_encounter_modes
 * selects SORTSWEEP).  A WHM ensemble whose Danby drift
 * fails for a massive body returns SWG_ERR_DRIFT from the step call (the reference stops
 * the run). */
typedef struct swg_ensemble swg_ensemble;
int swg_ensemble_create(swg_ctx *ctx, int integrator, int32_t nsys, const int32_t *npl, const int32_t *ntp,
                        swg_ensemble **ens);
int swg_ensemble_destroy(swg_ensemble *ens);
/* per-system central body: GMcb[nsys], Rcb[nsys] (Rcb may be NULL) */
int swg_ensemble_set_cb(swg_ensemble *ens, const double *GMcb, const double *Rcb);
int swg_ensemble_set_pl(swg_ensemble *ens, const double *rh, const double *vh, const double *Gmass,
                        const double *radius, const double *rhill);
int swg_ensemble_set_tp(swg_ensemble *ens, const double *rh, const double *vh);
int swg_ensemble_set_param(swg_ensemble *ens, double dt, double rhscale, int lclose, int precision);
/* SyMBA: modes of the level-0 pl-pl and pl-tp checks (param%lencounter_sas_plpl / _pltp),
 * SWG_ENC_TRIANGULAR (default) or SWG_ENC_SORTSWEEP: one radix sort of every system's
 * bounding-box extents, each body sweeping its own system's run; each system's list is the
 * one encounter_check_all_plpl / _pltp returns for it alone in that mode. */
int swg_ensemble_set_encounter_modes(swg_ensemble *ens, int enc_plpl, int enc_pltp);
/* GMTINY of param%GMTINY (swiftest_io.f90 param reader, symba_util.f90:175-208): in a SyMBA
 * ensemble, the bodies of a system with Gmass below gmtiny (which must follow the others in
 * its block, as Gmass-descending order leaves them) are semi-interacting: pairs of two of them
 * are left out of the pl-pl kick and the pl-pl level-0 check, each system's count of fully
 * interacting bodies fixed at swg_ensemble_initialize (call this before it; 0 = none).  Such
 * ensembles take the TRIANGULAR pl-pl check and the mixed path's broadcast pl-pl kernel. */
int swg_ensemble_set_gmtiny(swg_ensemble *ens, double gmtiny);
int swg_ensemble_initialize(swg_ensemble *ens);
int swg_ensemble_step(swg_ensemble *ens, int32_t nsteps);
int swg_ensemble_get_pl(swg_ensemble *ens, double *rh, double *vh, int32_t *status);
int swg_ensemble_get_tp(swg_ensemble *ens, double *rh, double *vh, int32_t *status);
/* swg_system_get_pl_masses of every system (NPL values each, CSR order). */
int swg_ensemble_get_pl_masses(swg_ensemble *ens, double *Gmass, double *radius, double *rhill);
/* out[9*nsys]: per system the nine values of swg_system_energy */
int swg_ensemble_energy(swg_ensemble *ens, double *out);
/* out[4*nsys]: per system the four values of swg_system_collision_terms */
int swg_ensemble_collision_terms(swg_ensemble *ens, double *out);
/* out[6] over all systems: system-steps with encounters, max recursion depth, sum plpl
 * enc, sum pltp enc, collisions, recursion sub-steps */
int swg_ensemble_stats(swg_ensemble *ens, int64_t *out);
/* level-0 pl-pl list of system sys from the last step, indices local to the system */
int swg_ensemble_plpl_list(swg_ensemble *ens, int32_t sys, int64_t cap, int64_t *n, int32_t *i1, int32_t *i2);
/* The state exchange and the first-step flags of every system, as for single systems
 * (swg_system_set_state, swg_system_reset_first_step). */
int swg_ensemble_set_state(swg_ensemble *ens, const double *rh, const double *vh, const double *trh,
                           const double *tvh);
int swg_ensemble_get_state_async(swg_ensemble *ens, double *rh, double *vh, double *trh, double *tvh);
int swg_ensemble_reset_first_step(swg_ensemble *ens);
/* WHM and HELIO ensembles replay each step as a CUDA graph captured after the first step
 * (default on; results are identical either way).  SyMBA steps always run eagerly: each
 * takes one host decision (the encounter-list sizes). */
int swg_ensemble_use_graphs(swg_ensemble *ens, int enable);
/* Kernel of the batched mixed-precision kick (no counterpart in the reference).  By
 * default (variant -1) the pl-pl kick evaluates each pair once for both bodies
 * (SWG_KICK_SYMMETRIC) and the pl-tp kick takes the fastest of SWG_KICK_NVARIANT tile
 * shapes of the receiver-broadcast kernel for its GPU and mean system size, timed on the
 * ensemble's own data at its first kick and cached in $SWG_TUNE_CACHE, else
 * $HOME/.cache/swiftest_gb300/kick_tune.txt.  Every broadcast shape gives bit-identical
 * accelerations; the symmetric kernel adds the same terms in another order.  Variants
 * 0 .. SWG_KICK_NVARIANT-1 force that broadcast shape on both kinds.  kick_variant reads
 * the kernel in use for kind 0 (pl-pl) or 1 (pl-tp), -1 before the first mixed kick of
 * that kind, with kind 2 the symmetric kick's strip length, with kind 3 its warps per
 * block and with kind 4 its bodies per tile. */
#define SWG_KICK_NVARIANT 5
#define SWG_KICK_SYMMETRIC 5
int swg_ensemble_set_kick_variant(swg_ensemble *ens, int variant);
/* Strip length of the symmetric pl-pl kick: each work item evaluates one row tile against
 * `strip` tile pairs, and a body's sums are split into one slot per item, so the strip sets
 * how the terms are grouped (results within the mixed-kick tolerance of each other, each
 * deterministic).  By default (0) the strips 1, 2, 4, 8 and 16 are timed on the ensemble's
 * own data at its first mixed kick (the minimum of five launches each) and the default 4 is
 * kept unless another is more than 3% faster; the choice is cached like the tile shapes.
 * 1, 2, 4, 8 or 16 forces it.  swg_ensemble_kick_variant with kind 2 reads the strip in use (-1 before the first
 * mixed kick). */
int swg_ensemble_set_kick_strip(swg_ensemble *ens, int strip);
/* Warps per block of the symmetric pl-pl kick (no counterpart in the reference).  Every warp
 * is an independent worker of the persistent grid, so 1, 2 and 4 give the same bits; by
 * default (0) the autotuner times the three at the chosen strip and keeps one warp unless
 * another count is more than 3% faster (cached with the strip).  1, 2 or 4 forces it;
 * swg_ensemble_kick_variant with kind 3 reads the count in use (-1 before the first mixed
 * kick). */
int swg_ensemble_set_kick_warps(swg_ensemble *ens, int warps);
/* Bodies per tile of the symmetric pl-pl kick (no counterpart in the reference): 128 (four
 * receivers per lane) or 64 (two; one warp per block).  The tile decides how a body's sums
 * are split into slots, so the two agree within the mixed-kick tolerance, each
 * deterministic.  By default (0) the autotuner times both (each at its default strip) before
 * the strip and keeps 128 unless 64 is more than 3% faster (cached with the strip);
 * swg_ensemble_kick_variant with kind 4 reads the tile in use (-1 before the first mixed
 * kick). */
int swg_ensemble_set_kick_tile(swg_ensemble *ens, int tile);
/* Tiles per row group of the symmetric pl-pl kick (no counterpart in the reference), 128-body
 * tiles only: with 2 or 4, a block of that many warps takes each item, one receiver tile per
 * warp against a strip of tiles J in step, and adds the warps' partner sums of each J in
 * warp order into one pair slot per group instead of one per tile: fewer slot bytes written
 * and read back.  The sums are grouped differently from one-row items (1), so results agree
 * within the mixed-kick tolerance, each deterministic.  By default (0) the autotuner times
 * groups 2 and 4 at strips 2 and 4 after the one-row shapes and takes the fastest group
 * only when it is more than 3% faster than the best one-row shape (cached with the strip); a
 * forced warps-per-block count or 64-body tile keeps one-row items, and a forced group of 2
 * or 4 takes 128-body tiles unless the tile is forced.  1, 2 or 4 forces it;
 * swg_ensemble_kick_variant with kind 5 reads the group in use (-1 before the first mixed
 * kick; kind 3 then reads the group's block size). */
int swg_ensemble_set_kick_group(swg_ensemble *ens, int group);
/* swiftest_kick_getacch_int_all_tri_pl (swiftest_kick.f90:183-264) of every system from its
 * current positions, in the ensemble's precision and pair rule (radius guard for SyMBA or
 * with close-encounter checks): acc[3*NPL] on the host, zero-based sums over all pairs. */
int swg_ensemble_getacch_int_pl(swg_ensemble *ens, double *acc);
int swg_ensemble_kick_variant(swg_ensemble *ens, int kind, int *variant);
int swg_ensemble_profile(swg_ensemble *ens, int enable);
int swg_ensemble_profile_read(swg_ensemble *ens, double *out);

/* ---- measurement helpers (no counterpart in the reference) ------------------------
 * Per-kernel-class CUDA-event profile of the step loop: classes 0 pl-pl kick,
 * 1 pl-tp kick, 2 drift, 3 level-0 encounter checks, 4 SyMBA recursion lists.
 * out[2k] = launches recorded, out[2k+1] = summed milliseconds. */
int swg_system_profile(swg_system *sys, int enable);
int swg_system_profile_read(swg_system *sys, double *out);
/* write `bytes` of a context-owned buffer on the context stream (evicts L2) */
int swg_flush_l2(swg_ctx *ctx, int64_t bytes);
/* CUDA events on the context stream: 16 slots */
int swg_event_record(swg_ctx *ctx, int slot);
int swg_event_elapsed(swg_ctx *ctx, int a, int b, double *ms);
/* FMA-chain throughput probe: kind 0 FP32 (FFMA), 1 FP64 (DFMA), 2 packed FP32 pairs
 * (fma.rn.f32x2, two FMAs per lane and instruction); TFLOP/s */
int swg_probe_peak(swg_ctx *ctx, int kind, double *tflops);

#ifdef __cplusplus
}
#endif
#endif
