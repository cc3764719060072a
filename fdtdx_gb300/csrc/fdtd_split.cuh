// CPML corrections of a split half-step (sm_103a).
//
// The split form of a forward half-step runs the plain TMA kernel over the whole grid (the
// Yee update with the bare curl, every cell; the zero halo comes from the TMA fill), then
// adds the CPML terms of each slab cell in separate launches, one per axis: psi advanced
// from the slab-axis differences and the two curl components that axis corrects updated.
// The update is linear in the curl, so
//   E_new = E + s c m (curl + dcurl) / (1 + q) = [plain update] + s c m dcurl / (1 + q),
// with the fused shell kernel's terms (ax_term: fdtdx/core/physics/curl.py:284-308,
// fdtdx/objects/boundaries/perfectly_matched_layer.py:138-190) and its update factors
// (s = +1 and q = c sigma eta0 m / 2 for E, s = -1 and q = c sigma m / (2 eta0) for H).
// Results differ from the fused kernels only by rounding.  The axes run in x, y, z order,
// as the fused kernels add them, so a cell in two or three slabs (an edge or a corner) sees
// its corrections one launch after another; the two slabs of an axis are disjoint.
//
// A reverse step (fdtdx/fdtd/update.py:751-807 inverting the update with psi frozen) splits
// the same way: E_old = [(1 + q) E - s c m curl] / (1 - q) = [plain reverse] - s c m dcurl /
// (1 - q), dcurl from the stored psi, which the reverse step does not advance.
//
// One thread per slab cell in psi order (a slab's psi array is dense over the slab box), so
// psi is read (and, forward, written) with unit stride.  Needs the per-axis slab table of a
// scene without a periodic axis (zero halo, UpdArgs::axt == 2).
#pragma once
#include "fdtd_kernels.cuh"

namespace fdtd {

template <bool REV, bool HSIDE, int AX>
__global__ void __launch_bounds__(256) k_pml_corr(const __grid_constant__ UpdArgs a) {
    const int side = blockIdx.y;
    const DSlab& sl = a.axs[AX][side];
    const int L = sl.L;
    if (L == 0) return;
    const long long n = (long long)sl.sx * sl.sy * sl.sz;
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    const Geo& g = a.g;
    // (i, j, k) of psi entry q: dims (sx, sy, sz), the slab axis offset by the slab's origin
    const int z = (int)(q % sl.sz);
    const long long r = q / sl.sz;
    const int y = (int)(r % sl.sy);
    const int x = (int)(r / sl.sy);
    const int i = AX == 0 ? x + sl.lo : x, j = AX == 1 ? y + sl.lo : y, k = AX == 2 ? z + sl.lo : z;
    const int l = AX == 0 ? x : (AX == 1 ? y : z);
    const long long N = g.N;
    const long long c = cell_index(g, i, j, k);
    // the slab-axis differences: d1 of component (AX + 2) % 3, d2 of component (AX + 1) % 3
    // (E step: backward differences of H; H step: forward differences of E; zero halo)
    constexpr int C1 = (AX + 2) % 3, C2 = (AX + 1) % 3;
    const long long step = AX == 0 ? (long long)g.ny * g.nz : (AX == 1 ? (long long)g.nz : 1);
    const int pos = AX == 0 ? i : (AX == 1 ? j : k);
    const int ext = AX == 0 ? g.nx : (AX == 1 ? g.ny : g.nz);
    const float* __restrict__ F = a.F;
    const float f1 = __ldg(F + C1 * N + c), f2 = __ldg(F + C2 * N + c);
    float d1, d2;
    if (HSIDE) {
        const bool in = pos + 1 < ext;
        d1 = (in ? __ldg(F + C1 * N + c + step) : 0.f) - f1;
        d2 = (in ? __ldg(F + C2 * N + c + step) : 0.f) - f2;
    } else {
        const bool in = pos > 0;
        d1 = f1 - (in ? __ldg(F + C1 * N + c - step) : 0.f);
        d2 = f2 - (in ? __ldg(F + C2 * N + c - step) : 0.f);
    }
    const float* co = sl.coef + (HSIDE ? 3 * L : 0);
    float* __restrict__ p1 = a.axp[AX][side][0];
    float* __restrict__ p2 = a.axp[AX][side][1];
    float q1 = p1[q], q2 = p2[q];
    if (!REV) {
        const float ca = __ldg(co + l), cb = __ldg(co + L + l);
        q1 = cb * q1 + ca * d1;
        q2 = cb * q2 + ca * d2;
        p1[q] = q1;
        p2[q] = q2;
    }
    float c1 = q1, c2 = q2;
    if (!sl.kappa_one) {
        const float ikm1 = __ldg(co + 2 * L + l) - 1.f;
        c1 = ikm1 * d1 + q1;
        c2 = ikm1 * d2 + q2;
    }
    // curl component (AX + 1) % 3 gets -c1, component (AX + 2) % 3 gets +c2
    const int wall = HSIDE ? g.pmc : g.pec;
    const float s = (HSIDE != REV) ? -g.c : g.c;
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int comp = t == 0 ? C2 : C1;
        const float dc = t == 0 ? -c1 : c2;
        if (wall && face_zero(g, wall, comp, i, j, k)) continue;
        const float m = a.mat ? __ldg(a.mat + (a.n_mat == 3 ? comp * N : 0) + c) : a.mat_scalar;
        float f = s * m * dc;
        if (a.sig) {
            const float sg = __ldg(a.sig + (a.n_sig == 3 ? comp * N : 0) + c);
            const float qs = HSIDE ? g.c * sg / g.eta0 * m / 2.f : g.c * sg * g.eta0 * m / 2.f;
            f /= REV ? 1.f - qs : 1.f + qs;
        }
        a.Uout[comp * N + c] += f;
    }
}

}  // namespace fdtd
