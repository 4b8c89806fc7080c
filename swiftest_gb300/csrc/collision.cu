// collision.cu -- host-side resolution of the collisions the SyMBA recursion detects.
//
// The reference detects collisions inside the recursion (collision_check_plpl / _pltp,
// src/collision/collision_check.f90:60-271; on the GPU: blk_collision_check in
// symba_dev.cuh) and resolves them on the host between two recursion sub-steps
// (collision_resolve_plpl / _pltp, src/collision/collision_resolve.f90:521-695).  Here the
// device recursion pauses at that point, the host runs the resolution below on copies of
// the system's arrays, and the recursion resumes.
//
// pl-pl: collision_resolve_plpl with the MERGE model (collision_generate_merge,
// src/collision/collision_generate.f90:158-260; collision_resolve_mergeaddsub,
// collision_resolve.f90:326-518) and the parts of swiftest_util_rearray_pl
// (src/swiftest/swiftest_util.f90:1638-1808) that change the state.  Energy tracking is on
// (as in runs that report |dE/E|), and masses are G*m (the reference's m = G*m/GU with
// GU = 1): energies and angular momenta are G times the reference's, every ratio is the
// same.  Per resolution:
//   1. sync: the central body's barycentric velocity (vb2vh, reverse order; the bodies'
//      vh are not refreshed after this, the merged ones get theirs from b2h) and position
//      (rh2rb, which also gives every body's rb);
//   2. E_before, L_before: the system's energy and angular momentum
//      (swiftest_util_get_energy_and_momentum_system, swiftest_util.f90:1172-1401); its
//      O(N^2) pairwise potential is formed on the device (k_pot_terms, k_pot_rowsum: each
//      row added in ascending j), the rows and the O(N) terms are added here in index order;
//   3. each COLLIDED pair whose two bodies were both flagged by the check, in list order:
//      the impactors' centre of mass (rb = rh + cb rb), the angular momentum of each impactor
//      about it, L_escape += both (no rotation: the reference books the pre-collision
//      orbital angular momentum as escaped), the merged body at the centre of mass with the
//      summed G*m and the radius of the summed volume, its velocity torqued by the
//      impactors' angular momentum (collision_util_velocity_torque,
//      collision_util.f90:1001-1026), list entries of the removed body redirected to the
//      merged one (a resulting self-pair becomes INACTIVE);
//   4. the Hill radius of every body from its current orbit (set_rhill in rearray,
//      swiftest_util.f90:2260-2280, with the semimajor axis of swiftest_orbel_xv2el);
//   5. the new system angular momentum: each merged body's velocity is torqued by
//      -(L_after - L_before) * m / (sum of the merged masses), then E_collisions +=
//      E_after - E_before (E_before stays the value of step 2 through a cascade, as in the
//      reference);
//   6. the cascade: the pl-pl list is checked again at the same level and with the level's
//      step (newly collided pairs flag their bodies, cb rb and rb are recomputed); repeat
//      from 3 while any pair collides, at most 1000 times.
// A velocity change at the merged body's position cannot restore the component of the
// impactors' angular momentum along that position, so, as in the reference, the system's
// angular momentum changes by that radial component at each merge (less than the L_escape
// booked for it).
// Bodies leave the system in place rather than by re-arraying: the merged body keeps the
// slot of the more massive impactor (the first on a tie, as maxloc picks it); the other
// keeps its slot with status INACTIVE, zero G*m, radius, Hill radius and velocity and a
// distant position of its own, so it exerts no force, is neither kicked nor drifted, and
// never meets an encounter radius.  Not restated: the re-sort by mass and the re-run of
// the encounter checks inside rearray (whose old and new lists are matched entry by entry),
// and the kinship grouping of a body that collides with two others in one check (the
// reference merges all three at once; here the first pair merges, the other pair is set
// ACTIVE again and merges in the cascade if it still collides).
// pl-tp: the test particle of every collided pair is discarded (collision_resolve_pltp).
// The OpenMP sums of the reference are taken in index order.  This file is compiled with
// -ffp-contract=off on the host and -fmad=false on the device, so the arithmetic is the C
// oracle's, bit for bit.
#include <cmath>
#include <cstdint>
#include <vector>

#include "collision_one.cuh"
#include "swg_internal.cuh"

namespace swg {

namespace {

constexpr double DP_TINY = 2.2250738585072014e-308;  // tiny(1.0_DP)
constexpr double DP_EPS = 2.220446049250313e-16;     // epsilon(1.0_DP)
constexpr double PI = 3.141592653589793238462643383279502884197;
constexpr double THIRD = 0.333333333333333333333333333333333333333;
constexpr int MAXCASCADE = 1000;  // collision_resolve.f90:543

// gfortran NORM2 (used by the operators .mag. and .unit.)
double norm2_3(const double *x) { return hd_norm2_3(x[0], x[1], x[2]); }

// ---- the O(N^2) part of the resolution's energies on the device
// Term (i, j) of the pairwise potential for i < j < n, j in [j0, j1), at
// terms[(j - j0) * n + i]; zero where either body is INACTIVE (adding +0.0 to a row that
// starts at +0.0 and only gains negative terms leaves it unchanged, as skipping does).
__global__ void __launch_bounds__(128) k_pot_terms(int n, int j0, int j1, const double *__restrict__ rb,
                                                   const double *__restrict__ Gm, const int32_t *__restrict__ st,
                                                   double *__restrict__ terms) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int j = j0 + (int)blockIdx.y;
    if (i >= n || j >= j1 || i >= j) return;
    const bool on = st[i] != ST_INACTIVE && st[j] != ST_INACTIVE;
    terms[(size_t)(j - j0) * n + i] = on ? hd_pot_term(rb + 3 * (size_t)i, rb + 3 * (size_t)j, Gm[i], Gm[j]) : 0.0;
}
// Row i of the potential, one thread per row: the terms added in ascending j (the
// reference's sum(pepl(i+1:npl)), swiftest_util.f90:1386), continued over j chunks.
__global__ void __launch_bounds__(32) k_pot_rowsum(int n, int j0, int j1, const double *__restrict__ terms,
                                                   double *__restrict__ rows) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double r = j0 == 0 ? 0.0 : rows[i];
    int j = j0 > i + 1 ? j0 : i + 1;
    const double *t = terms + (size_t)(j - j0) * n + i;
    for (; j + 8 <= j1; j += 8, t += 8 * (size_t)n) {
        double v[8];
#pragma unroll
        for (int k = 0; k < 8; k++) v[k] = t[(size_t)k * n];
#pragma unroll
        for (int k = 0; k < 8; k++) r = r + v[k];
    }
    for (; j < j1; j++, t += n) r = r + *t;
    rows[i] = r;
}

// rows[i] = sum over j > i of the potential terms, computed on c's device (scratch slot 23)
int device_pot_rows(swg_ctx *c, int n, const double *rb, const double *Gm, const int32_t *st, double *rows) {
    if (n <= 0) return SWG_OK;
    const size_t un = (size_t)n;
    const size_t J = std::max<size_t>(1, std::min<size_t>(std::min<size_t>(un, ((size_t)16 << 20) / un), 65535));
    const size_t head = 5 * un * sizeof(double) + ((un * sizeof(int32_t) + 255) & ~(size_t)255);
    void *p = nullptr;
    SWG_TRY(ensure_slot(c, 23, head + J * un * sizeof(double), &p));
    double *drb = (double *)p, *dGm = drb + 3 * un, *drows = dGm + un;
    int32_t *dst = (int32_t *)(drows + un);
    double *terms = (double *)((char *)p + head);
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(drb, rb, 3 * un * sizeof(double), cudaMemcpyHostToDevice, c->stream), "pot"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(dGm, Gm, un * sizeof(double), cudaMemcpyHostToDevice, c->stream), "pot"));
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(dst, st, un * sizeof(int32_t), cudaMemcpyHostToDevice, c->stream), "pot"));
    for (size_t j0 = 0; j0 < un; j0 += J) {
        const size_t j1 = std::min(un, j0 + J);
        k_pot_terms<<<dim3((unsigned)((un + 127) / 128), (unsigned)(j1 - j0)), 128, 0, c->stream>>>(
            n, (int)j0, (int)j1, drb, dGm, dst, terms);
        c->launches++;
        SWG_TRY(launch_status(c, "pot_terms"));
        k_pot_rowsum<<<(unsigned)((un + 31) / 32), 32, 0, c->stream>>>(n, (int)j0, (int)j1, terms, drows);
        c->launches++;
        SWG_TRY(launch_status(c, "pot_rowsum"));
    }
    SWG_TRY(cuda_status(c, cudaMemcpyAsync(rows, drows, un * sizeof(double), cudaMemcpyDeviceToHost, c->stream), "pot"));
    return cuda_status(c, cudaStreamSynchronize(c->stream), "pot");
}

// operator .unit. (src/operator/operator_unit.f90)
void unit3(const double *a, double *u) {
    const double m = norm2_3(a);
    for (int d = 0; d < 3; d++) u[d] = m > DP_TINY ? a[d] / m : 0.0;
}

// operator .cross. (src/operator/operator_cross.f90)
void cross3(const double *a, const double *b, double *c) {
    c[0] = a[1] * b[2] - a[2] * b[1];
    c[1] = a[2] * b[0] - a[0] * b[2];
    c[2] = a[0] * b[1] - a[1] * b[0];
}

// collision_util_velocity_torque (src/collision/collision_util.f90:1001-1026): a velocity
// change at r that adds the part of dL perpendicular to r to the body's angular momentum
void velocity_torque(const double *dL, double mass, const double *r, double *v) {
    double dLu[3], ru[3], q[3], c[3];
    unit3(dL, dLu);
    unit3(r, ru);
    const double rmag = norm2_3(r), vmag = norm2_3(v);
    for (int d = 0; d < 3; d++) q[d] = dL[d] / (rmag * mass);
    const double vapply_mag = norm2_3(q);
    if (vapply_mag / vmag > DP_EPS) {
        cross3(dLu, ru, c);
        for (int d = 0; d < 3; d++) v[d] = v[d] + vapply_mag * c[d];
    }
}

// swiftest_orbel_xv2el (src/swiftest/swiftest_orbel.f90:913-1072): the semimajor axis
double xv2el_a(double mu, const double *r, const double *v) {
    const double TINYV = 4.0e-15;  // swiftest_orbel.f90:11
    const double hx = r[1] * v[2] - r[2] * v[1], hy = r[2] * v[0] - r[0] * v[2], hz = r[0] * v[1] - r[1] * v[0];
    const double h2 = hx * hx + hy * hy + hz * hz;
    if (h2 <= 10.0 * DP_TINY) return 0.0;
    const double rr = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const double energy = 0.5 * v2 - mu / rr;
    if (std::fabs(energy * rr / mu) < std::sqrt(TINYV)) return 0.5 * h2 / mu;  // parabola
    const double a = -0.5 * mu / energy;
    if (a < 0.0 && !(-h2 / (mu * a) > TINYV)) return 0.5 * h2 / mu;  // parabola
    return a;
}

// a removed body's slot: no velocity, a distant position of its own (slot index k)
void park(double *r, double *v, int64_t k) {
    r[0] = 1.0e6 + (double)k;
    r[1] = r[2] = 0.0;
    v[0] = v[1] = v[2] = 0.0;
}

// The collision resolution's view of one system (host copies) and its work arrays.
struct Resolver {
    CollisionSystem &c;
    std::vector<double> rb, vh;
    std::vector<unsigned char> coll;
    double cbrb[3] = {0.0, 0.0, 0.0}, cbvb[3] = {0.0, 0.0, 0.0};

    std::vector<double> prow;  // rows of the pairwise potential
    bool dev_failed = false;

    explicit Resolver(CollisionSystem &cs)
        : c(cs), rb(3 * (size_t)std::max(cs.npl, 1)), vh(3 * (size_t)std::max(cs.npl, 1)),
          coll((size_t)std::max(cs.npl, 1), 0), prow((size_t)std::max(cs.npl, 1)) {}

    bool active(int32_t i) const { return c.status[i] != ST_INACTIVE; }

    // swiftest_util_coord_rh2rb_pl (swiftest_util.f90:488-521)
    void rh2rb() {
        double Gmtot = c.GMcb, xtmp[3] = {0.0, 0.0, 0.0};
        for (int32_t i = 0; i < c.npl; i++) {
            if (!active(i)) continue;
            Gmtot = Gmtot + c.Gm[i];
            for (int d = 0; d < 3; d++) xtmp[d] = xtmp[d] + c.Gm[i] * c.rh[3 * i + d];
        }
        for (int d = 0; d < 3; d++) cbrb[d] = -xtmp[d] / Gmtot;
        for (int32_t i = 0; i < c.npl; i++) {
            if (!active(i)) continue;
            for (int d = 0; d < 3; d++) rb[3 * i + d] = c.rh[3 * i + d] + cbrb[d];
        }
    }

    // swiftest_util_coord_vb2vh_pl (swiftest_util.f90:363-395)
    void vb2vh() {
        for (int d = 0; d < 3; d++) cbvb[d] = 0.0;
        for (int32_t b = c.npl - 1; b >= 0; b--) {
            if (!active(b)) continue;
            for (int d = 0; d < 3; d++) cbvb[d] = cbvb[d] - c.Gm[b] * c.vb[3 * b + d] / c.GMcb;
        }
        for (int32_t b = 0; b < c.npl; b++)
            for (int d = 0; d < 3; d++) vh[3 * b + d] = c.vb[3 * b + d] - cbvb[d];
    }

    // swiftest_util_get_energy_and_momentum_system with the triangular potential, as the
    // resolution calls it: no spin terms, cb rb/vb as the sync left them.  The potential's
    // rows (each added in ascending j) are formed on the device, the rows are added here in
    // index order; with_te = false leaves te unset and forms only L.
    void energy(double &te, double *L, bool with_te = true) {
        const double mcb = c.GMcb;
        const double kecb = mcb * (cbvb[0] * cbvb[0] + cbvb[1] * cbvb[1] + cbvb[2] * cbvb[2]);
        const double Lcb[3] = {mcb * (cbrb[1] * cbvb[2] - cbrb[2] * cbvb[1]),
                               mcb * (cbrb[2] * cbvb[0] - cbrb[0] * cbvb[2]),
                               mcb * (cbrb[0] * cbvb[1] - cbrb[1] * cbvb[0])};
        double kesum = 0.0, Lsum[3] = {0.0, 0.0, 0.0};
        for (int32_t i = 0; i < c.npl; i++) {
            if (!active(i)) continue;
            const double *r = &rb[3 * i], *v = &c.vb[3 * i];
            const double m = c.Gm[i];
            Lsum[0] = Lsum[0] + m * (r[1] * v[2] - r[2] * v[1]);
            Lsum[1] = Lsum[1] + m * (r[2] * v[0] - r[0] * v[2]);
            Lsum[2] = Lsum[2] + m * (r[0] * v[1] - r[1] * v[0]);
            kesum = kesum + m * (v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        }
        for (int d = 0; d < 3; d++) L[d] = Lcb[d] + Lsum[d];
        if (!with_te) return;
        if (!c.dev || device_pot_rows(c.dev, c.npl, rb.data(), c.Gm, c.status, prow.data()) != SWG_OK) {
            dev_failed = true;
            te = 0.0;
            return;
        }
        double pe = 0.0;
        for (int32_t i = 0; i < c.npl; i++)
            if (active(i)) pe = pe + prow[i];
        double pecb = 0.0, be = 0.0;
        for (int32_t i = 0; i < c.npl; i++) {
            if (!active(i)) continue;
            pecb = pecb + (-c.GMcb * c.Gm[i] / norm2_3(&rb[3 * i]));
            be = be + (-3.0 * c.Gm[i] * c.Gm[i] / (5.0 * c.R[i]));
        }
        pe = pe + pecb;
        const double ke = 0.5 * (kecb + kesum);
        te = ke + pe + be;
    }

    // collision_check_plpl (collision_check.f90:60-160) over the list at the resolution's
    // level: ACTIVE pairs whose index1 body sits at level >= irec
    bool check_plpl() {
        bool any = false;
        for (int64_t k = 0; k < c.npp; k++) {
            if (c.pp_st[k] != ST_ACTIVE) continue;
            const int32_t i = c.pp_i1[k] - 1, j = c.pp_i2[k] - 1;
            if (c.levelg[i] < c.irec) continue;
            double x[3], v[3];
            for (int d = 0; d < 3; d++) {
                x[d] = c.rh[3 * i + d] - c.rh[3 * j + d];
                v[d] = c.vb[3 * i + d] - c.vb[3 * j + d];
            }
            if (d_collision_one(x[0], x[1], x[2], v[0], v[1], v[2], c.Gm[i] + c.Gm[j], c.R[i] + c.R[j], c.dt,
                                         c.pp_lv[k] != 0)) {
                c.pp_st[k] = ST_COLLIDED;
                coll[i] = coll[j] = 1;
                any = true;
            }
        }
        return any;
    }

    // collision_generate_merge + collision_resolve_mergeaddsub for the pair (i, j):
    // returns the slot of the merged body
    int32_t merge(int32_t i, int32_t j) {
        const double m1 = c.Gm[i], m2 = c.Gm[j], mtot = m1 + m2;
        double rb1[3], rb2[3], rbcom[3], vbcom[3], rc1[3], rc2[3], vc1[3], vc2[3];
        const double *vb1 = &c.vb[3 * i], *vb2 = &c.vb[3 * j];
        for (int d = 0; d < 3; d++) {
            rb1[d] = c.rh[3 * i + d] + cbrb[d];
            rb2[d] = c.rh[3 * j + d] + cbrb[d];
        }
        for (int d = 0; d < 3; d++) {
            rbcom[d] = (m1 * rb1[d] + m2 * rb2[d]) / mtot;
            vbcom[d] = (m1 * vb1[d] + m2 * vb2[d]) / mtot;
        }
        for (int d = 0; d < 3; d++) {
            rc1[d] = rb1[d] - rbcom[d];
            rc2[d] = rb2[d] - rbcom[d];
            vc1[d] = vb1[d] - vbcom[d];
            vc2[d] = vb2[d] - vbcom[d];
        }
        const double L1[3] = {m1 * (rc1[1] * vc1[2] - rc1[2] * vc1[1]), m1 * (rc1[2] * vc1[0] - rc1[0] * vc1[2]),
                              m1 * (rc1[0] * vc1[1] - rc1[1] * vc1[0])};
        const double L2[3] = {m2 * (rc2[1] * vc2[2] - rc2[2] * vc2[1]), m2 * (rc2[2] * vc2[0] - rc2[0] * vc2[2]),
                              m2 * (rc2[0] * vc2[1] - rc2[1] * vc2[0])};
        double Lb[3];
        for (int d = 0; d < 3; d++) {
            Lb[d] = L1[d] + L2[d];
            c.L_escape[d] = c.L_escape[d] + L1[d] + L2[d];
        }
        const double Ri = c.R[i], Rj = c.R[j];
        const double volume = 4.0 / 3.0 * PI * (Ri * Ri * Ri + Rj * Rj * Rj);
        const double Rnew = std::pow(3.0 * volume / (4.0 * PI), THIRD);
        // the merged body carries no angular momentum about the centre of mass: the
        // residual 0 - Lb is torqued back onto its velocity
        double vnew[3] = {vbcom[0], vbcom[1], vbcom[2]};
        const double dL[3] = {-(0.0 - Lb[0]), -(0.0 - Lb[1]), -(0.0 - Lb[2])};
        velocity_torque(dL, mtot, rbcom, vnew);
        const int32_t keep = m2 > m1 ? j : i, gone = keep == i ? j : i;
        for (int d = 0; d < 3; d++) {  // b2h of the new body
            rb[3 * keep + d] = rbcom[d];
            c.rh[3 * keep + d] = rbcom[d] - cbrb[d];
            c.vb[3 * keep + d] = vnew[d];
            vh[3 * keep + d] = vnew[d] - cbvb[d];
        }
        c.Gm[keep] = mtot;
        c.R[keep] = Rnew;
        c.Gm[gone] = 0.0;
        c.R[gone] = 0.0;
        c.rhill[gone] = 0.0;
        c.status[gone] = ST_INACTIVE;
        c.lmask[gone] = 0;
        park(&c.rh[3 * (int64_t)gone], &c.vb[3 * (int64_t)gone], gone);
        coll[i] = coll[j] = 0;
        for (int64_t q = 0; q < c.npp; q++) {
            if (c.pp_i1[q] == gone + 1) c.pp_i1[q] = keep + 1;
            if (c.pp_i2[q] == gone + 1) c.pp_i2[q] = keep + 1;
            if (c.pp_i1[q] == c.pp_i2[q]) c.pp_st[q] = ST_INACTIVE;
        }
        for (int64_t q = 0; q < c.npt; q++)
            if (c.pt_i1[q] == gone + 1) c.pt_i1[q] = keep + 1;
        return keep;
    }

    // swiftest_util_set_rhill (swiftest_util.f90:2260-2280) of every body
    void set_rhill() {
        if (c.GMcb <= DP_TINY) return;
        for (int32_t b = 0; b < c.npl; b++) {
            if (!active(b)) continue;
            const double a = xv2el_a(c.GMcb + c.Gm[b], &c.rh[3 * b], &vh[3 * b]);
            const double scale = std::pow(c.Gm[b] / c.GMcb / 3.0, THIRD);
            c.rhill[b] = a > 0.0 ? a * scale : norm2_3(&c.rh[3 * b]) * scale;
        }
    }

    int64_t resolve_plpl() {
        bool any = false;
        for (int64_t k = 0; k < c.npp; k++) any |= c.pp_st[k] == ST_COLLIDED;
        if (!any) return 0;
        for (int64_t k = 0; k < c.npp; k++)
            if (c.pp_st[k] == ST_COLLIDED) coll[c.pp_i1[k] - 1] = coll[c.pp_i2[k] - 1] = 1;
        vb2vh();
        rh2rb();
        double E_before, L_before[3];
        energy(E_before, L_before);
        if (dev_failed) return -2;
        std::vector<int32_t> newb;
        int64_t nres = 0;
        for (int loop = 1;; loop++) {
            newb.clear();
            for (int64_t k = 0; k < c.npp; k++) {
                if (c.pp_st[k] != ST_COLLIDED) continue;
                const int32_t i = c.pp_i1[k] - 1, j = c.pp_i2[k] - 1;
                if (!coll[i] || !coll[j]) {  // one impactor already merged in this pass: test the pair again
                    if (active(i) && active(j) && i != j) c.pp_st[k] = ST_ACTIVE;
                    continue;
                }
                newb.push_back(merge(i, j));
                nres++;
            }
            if (newb.empty()) break;
            double mnew = 0.0;
            for (int32_t b : newb) mnew = mnew + c.Gm[b];
            set_rhill();
            double E_after, L_after[3], dL[3];
            energy(E_after, L_after, false);
            for (int d = 0; d < 3; d++) dL[d] = L_after[d] - L_before[d];
            for (int32_t b : newb) {
                const double t[3] = {-dL[0] * c.Gm[b] / mnew, -dL[1] * c.Gm[b] / mnew, -dL[2] * c.Gm[b] / mnew};
                velocity_torque(t, c.Gm[b], &rb[3 * b], &c.vb[3 * b]);
            }
            energy(E_after, L_after);
            if (dev_failed) return -2;
            c.E_collisions = c.E_collisions + (E_after - E_before);
            if (!check_plpl()) break;
            if (loop == MAXCASCADE) return -1;
            rh2rb();
        }
        return nres;
    }
};

}  // namespace

int64_t resolve_collisions_host(CollisionSystem &c) {
    Resolver r(c);
    const int64_t npp = r.resolve_plpl();
    if (npp < 0) return npp;
    // pl-tp: the test particle of every collided pair is discarded
    int64_t nres = npp;
    for (int64_t k = 0; k < c.npt; k++) {
        if (c.pt_st[k] != ST_COLLIDED) continue;
        const int32_t j = c.pt_i2[k] - 1;
        if (c.tstatus[j] == ST_INACTIVE) continue;
        c.tstatus[j] = ST_INACTIVE;
        c.tlmask[j] = 0;
        park(&c.trh[3 * (int64_t)j], &c.tvb[3 * (int64_t)j], (int64_t)c.npl + j);
        nres++;
    }
    return nres;
}

}  // namespace swg
