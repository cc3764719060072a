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

// The z-slab corrections two cells per thread: a z slab's rows are L cells long and
// contiguous in the field arrays, so with L, the slab origin and nz even (and 8-byte aligned
// arrays) each thread loads and stores float2 pairs and shares the difference between its two
// cells.  Same arithmetic as k_pml_corr<REV, HSIDE, 2>, cell by cell.
template <bool REV, bool HSIDE>
__global__ void __launch_bounds__(256) k_pml_corr_z2(const __grid_constant__ UpdArgs a) {
    const int side = blockIdx.y;
    const DSlab& sl = a.axs[2][side];
    const int L = sl.L;
    if (L == 0) return;
    const long long n2 = (long long)sl.sx * sl.sy * sl.sz / 2;
    const long long q2 = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q2 >= n2) return;
    const long long q = 2 * q2;
    const Geo& g = a.g;
    const int l = (int)(q % sl.sz);  // even
    const long long r = q / sl.sz;
    const int j = (int)(r % sl.sy);
    const int i = (int)(r / sl.sy);
    const int k = l + sl.lo;  // even: the pair is (k, k + 1)
    const long long N = g.N;
    const long long c = cell_index(g, i, j, k);
    constexpr int C1 = 1, C2 = 0;  // (AX + 2) % 3, (AX + 1) % 3 for AX = 2
    const float* __restrict__ F = a.F;
    const float2 f1 = *reinterpret_cast<const float2*>(F + C1 * N + c);
    const float2 f2 = *reinterpret_cast<const float2*>(F + C2 * N + c);
    float d1[2], d2[2];
    if (HSIDE) {  // forward differences: (k + 1) - k, (k + 2) - (k + 1)
        const bool in = k + 2 < g.nz;
        d1[0] = f1.y - f1.x;
        d2[0] = f2.y - f2.x;
        d1[1] = (in ? __ldg(F + C1 * N + c + 2) : 0.f) - f1.y;
        d2[1] = (in ? __ldg(F + C2 * N + c + 2) : 0.f) - f2.y;
    } else {      // backward differences: k - (k - 1), (k + 1) - k
        const bool in = k > 0;
        d1[0] = f1.x - (in ? __ldg(F + C1 * N + c - 1) : 0.f);
        d2[0] = f2.x - (in ? __ldg(F + C2 * N + c - 1) : 0.f);
        d1[1] = f1.y - f1.x;
        d2[1] = f2.y - f2.x;
    }
    const float* co = sl.coef + (HSIDE ? 3 * L : 0);
    float2* p1 = reinterpret_cast<float2*>(a.axp[2][side][0] + q);
    float2* p2 = reinterpret_cast<float2*>(a.axp[2][side][1] + q);
    const float2 pv1 = *p1, pv2 = *p2;
    float q1[2] = {pv1.x, pv1.y}, q2v[2] = {pv2.x, pv2.y};
    float c1[2], c2[2];
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        if (!REV) {
            const float ca = __ldg(co + l + e), cb = __ldg(co + L + l + e);
            q1[e] = cb * q1[e] + ca * d1[e];
            q2v[e] = cb * q2v[e] + ca * d2[e];
        }
        c1[e] = q1[e];
        c2[e] = q2v[e];
        if (!sl.kappa_one) {
            const float ikm1 = __ldg(co + 2 * L + l + e) - 1.f;
            c1[e] = ikm1 * d1[e] + q1[e];
            c2[e] = ikm1 * d2[e] + q2v[e];
        }
    }
    if (!REV) {
        *p1 = make_float2(q1[0], q1[1]);
        *p2 = make_float2(q2v[0], q2v[1]);
    }
    const int wall = HSIDE ? g.pmc : g.pec;
    const float s = (HSIDE != REV) ? -g.c : g.c;
#pragma unroll
    for (int t = 0; t < 2; ++t) {
        const int comp = t == 0 ? C2 : C1;
        float2* U = reinterpret_cast<float2*>(a.Uout + comp * N + c);
        float2 u = *U;
        float* uv = reinterpret_cast<float*>(&u);
#pragma unroll
        for (int e = 0; e < 2; ++e) {
            if (wall && face_zero(g, wall, comp, i, j, k + e)) continue;
            const float dc = t == 0 ? -c1[e] : c2[e];
            const float m = a.mat ? __ldg(a.mat + (a.n_mat == 3 ? comp * N : 0) + c + e) : a.mat_scalar;
            float f = s * m * dc;
            if (a.sig) {
                const float sg = __ldg(a.sig + (a.n_sig == 3 ? comp * N : 0) + c + e);
                const float qs = HSIDE ? g.c * sg / g.eta0 * m / 2.f : g.c * sg * g.eta0 * m / 2.f;
                f /= REV ? 1.f - qs : 1.f + qs;
            }
            uv[e] += f;
        }
        *U = u;
    }
}

}  // namespace fdtd
