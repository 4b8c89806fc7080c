// collision.cu -- host-side resolution of the collisions the SyMBA recursion detects.
//
// The reference detects collisions inside the recursion (collision_check_plpl / _pltp,
// src/collision/collision_check.f90:60-271; on the GPU: blk_collision_check in
// symba_dev.cuh) and resolves them on the host between two recursion sub-steps
// (collision_resolve_plpl / _pltp, src/collision/collision_resolve.f90:521-695).  Here the
// device recursion pauses at that point, the host runs the resolution below on copies of
// the system's arrays, and the recursion resumes.  The collisional model is perfect
// merging (collision_generate_merge, src/collision/collision_generate.f90:158-260):
//   * pl-pl: the two bodies become one with the summed G*m, the radius of the summed
//     volume and the centre-of-mass position and velocity, kept in the slot of the more
//     massive body; its Hill radius is recomputed from the new orbit as
//     swiftest_util_set_rhill does (src/swiftest/swiftest_util.f90:2260-2280).
//   * pl-tp: the test particle is discarded.
// Bodies leave the system in place rather than by re-arraying: a removed body keeps its
// slot with status INACTIVE, zero mass, radius and Hill radius, no velocity and a distant
// position of its own, so it exerts no force, is neither kicked nor drifted, and never
// meets an encounter radius.  Encounter-list entries of a removed body are redirected to
// the merged body and a pair that becomes a self-pair is made INACTIVE, as the reference
// does with body ids.  Not restated: the angular-momentum torque on the merged body and
// the collision energy bookkeeping (E_collisions), cascades of new collisions within one
// resolution, and the re-sort of the arrays by mass.
#include <cmath>
#include <cstdint>

#include "swg_internal.cuh"

namespace swg {

namespace {

// swiftest_orbel_xv2aeq (src/swiftest/swiftest_orbel.f90:700-764), semimajor axis only
double xv2a(double mu, const double *r, const double *v) {
    const double TINYV = 4.0e-15;
    const double rr = std::sqrt(r[0] * r[0] + r[1] * r[1] + r[2] * r[2]);
    const double v2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
    const double hx = r[1] * v[2] - r[2] * v[1], hy = r[2] * v[0] - r[0] * v[2], hz = r[0] * v[1] - r[1] * v[0];
    const double h2 = hx * hx + hy * hy + hz * hz;
    if (h2 < 2.2250738585072014e-308) return 0.0;
    const double energy = 0.5 * v2 - mu / rr;
    if (std::fabs(energy * rr / mu) < std::sqrt(TINYV)) return 0.5 * h2 / mu;  // parabola
    const double a = -0.5 * mu / energy;
    if (a < 0.0) {
        const double fac = -h2 / (mu * a);
        if (!(fac > TINYV)) return 0.5 * h2 / mu;  // parabola
    }
    return a;
}

// a removed body's slot: no velocity, a distant position of its own (slot index k)
void park(double *r, double *v, int64_t k) {
    r[0] = 1.0e6 + (double)k;
    r[1] = r[2] = 0.0;
    v[0] = v[1] = v[2] = 0.0;
}

}  // namespace

int64_t resolve_collisions_host(CollisionSystem &c) {
    const double PI = 3.141592653589793238462643383279502884197;
    const double THIRD = 0.333333333333333333333333333333333333333;
    int64_t nres = 0;
    // pl-tp: the test particle of every collided pair is discarded
    for (int64_t k = 0; k < c.npt; k++) {
        if (c.pt_st[k] != ST_COLLIDED) continue;
        const int32_t j = c.pt_i2[k] - 1;
        if (c.tstatus[j] == ST_INACTIVE) continue;
        c.tstatus[j] = ST_INACTIVE;
        c.tlmask[j] = 0;
        park(&c.trh[3 * (int64_t)j], &c.tvb[3 * (int64_t)j], (int64_t)c.npl + j);
        nres++;
    }
    // pl-pl: merge in list order
    bool have_cbvb = false;
    double cbvb[3] = {0.0, 0.0, 0.0};
    for (int64_t k = 0; k < c.npp; k++) {
        if (c.pp_st[k] != ST_COLLIDED) continue;
        const int32_t i = c.pp_i1[k] - 1, j = c.pp_i2[k] - 1;
        if (i == j || c.status[i] == ST_INACTIVE || c.status[j] == ST_INACTIVE) continue;
        if (!have_cbvb) {  // the central body's velocity as swiftest_util_coord_vb2vh_pl sums it
            for (int32_t b = c.npl - 1; b >= 0; b--) {
                if (c.status[b] == ST_INACTIVE) continue;
                for (int d = 0; d < 3; d++) cbvb[d] = cbvb[d] - c.Gm[b] * c.vb[3 * b + d] / c.GMcb;
            }
            have_cbvb = true;
        }
        const int32_t keep = c.Gm[j] > c.Gm[i] ? j : i, gone = keep == i ? j : i;
        const double Gi = c.Gm[i], Gj = c.Gm[j], Gtot = Gi + Gj;
        double rnew[3], vnew[3], vh[3];
        for (int d = 0; d < 3; d++) {
            rnew[d] = (Gi * c.rh[3 * i + d] + Gj * c.rh[3 * j + d]) / Gtot;
            vnew[d] = (Gi * c.vb[3 * i + d] + Gj * c.vb[3 * j + d]) / Gtot;
            vh[d] = vnew[d] - cbvb[d];
        }
        const double volume = 4.0 / 3.0 * PI * (c.R[i] * c.R[i] * c.R[i] + c.R[j] * c.R[j] * c.R[j]);
        const double Rnew = std::pow(3.0 * volume / (4.0 * PI), THIRD);
        const double a = xv2a(c.GMcb + Gtot, rnew, vh);
        const double scale = std::pow(Gtot / c.GMcb / 3.0, THIRD);
        const double rhill = a > 0.0 ? a * scale : std::sqrt(rnew[0] * rnew[0] + rnew[1] * rnew[1] + rnew[2] * rnew[2]) * scale;
        for (int d = 0; d < 3; d++) {
            c.rh[3 * keep + d] = rnew[d];
            c.vb[3 * keep + d] = vnew[d];
        }
        c.Gm[keep] = Gtot;
        c.R[keep] = Rnew;
        c.rhill[keep] = rhill;
        c.Gm[gone] = 0.0;
        c.R[gone] = 0.0;
        c.rhill[gone] = 0.0;
        c.status[gone] = ST_INACTIVE;
        c.lmask[gone] = 0;
        park(&c.rh[3 * (int64_t)gone], &c.vb[3 * (int64_t)gone], gone);
        for (int64_t q = 0; q < c.npp; q++) {
            if (c.pp_i1[q] == gone + 1) c.pp_i1[q] = keep + 1;
            if (c.pp_i2[q] == gone + 1) c.pp_i2[q] = keep + 1;
            if (c.pp_i1[q] == c.pp_i2[q]) c.pp_st[q] = ST_INACTIVE;
        }
        for (int64_t q = 0; q < c.npt; q++)
            if (c.pt_i1[q] == gone + 1) c.pt_i1[q] = keep + 1;
        nres++;
    }
    return nres;
}

}  // namespace swg
