// Forward and time-reversed Yee half-steps, source injection, detector
// accumulation and PML-interface recording for the GB300 (sm_103a).
//
// One thread owns one cell of the updated field; the grid is
// (ceil(nz/32), ceil(ny/8), nx) with 32 threads along z, so every warp reads and
// writes 128 contiguous bytes per component.  Neighbour values of the
// differentiated field come from the L1/L2 (the planes i-1 / i+1 were touched by
// the previous / next z-blocks of the same block row a few microseconds apart).
// The CPML correction of a cell is fused into its half-step: a slab is tested by
// one unsigned compare per slab, so interior cells pay six compares.
#pragma once
#include "fdtd_device.cuh"

namespace fdtd {

// CPML correction of one cell (fdtdx/core/physics/curl.py:284-308, 371-394;
// fdtdx/objects/boundaries/perfectly_matched_layer.py:138-190).  d[] holds the six raw
// differences in the order (dy Fz, dz Fy, dz Fx, dx Fz, dx Fy, dy Fx); for a slab on axis a
// d_a F_j and d_a F_i are (3, 4), (5, 0), (1, 2) and the corrections go to
// curl[(a+1)%3] (minus) and curl[(a+2)%3] (plus).  psi is fetched by psi_fetch before the
// differences are formed, so its scattered slab reads overlap the field loads.
struct PsiPre {
    float v[FDTD_MAX_SLABS][2];
};

__device__ __forceinline__ long long psi_offset(const DSlab& sl, int i, int j, int k) {
    return ((long long)(i - (sl.axis == 0 ? sl.lo : 0)) * sl.sy + (j - (sl.axis == 1 ? sl.lo : 0))) * sl.sz +
           (k - (sl.axis == 2 ? sl.lo : 0));
}

__device__ __forceinline__ void psi_fetch(const UpdArgs& a, int i, int j, int k, PsiPre& pr, int active = 63) {
    const int idx3[3] = {i, j, k};
#pragma unroll
    for (int s = 0; s < FDTD_MAX_SLABS; ++s) {
        pr.v[s][0] = 0.f;
        pr.v[s][1] = 0.f;
        if (s >= a.n_slab || !(active >> s & 1)) continue;
        const DSlab& sl = a.slab[s];
        const int l = idx3[sl.axis] - sl.lo;
        if ((unsigned)l >= (unsigned)sl.L) continue;
        const long long p = psi_offset(sl, i, j, k);
        pr.v[s][0] = a.psi1[s][p];
        pr.v[s][1] = a.psi2[s][p];
    }
}

// cpml_correct with the psi values taken from a prefetch.
template <bool REV, bool HSIDE>
__device__ __forceinline__ void cpml_apply(const UpdArgs& a, int i, int j, int k, const float d[6], float cu[3],
                                           const PsiPre& pr, int active = 63) {
    const int idx3[3] = {i, j, k};
#pragma unroll
    for (int s = 0; s < FDTD_MAX_SLABS; ++s) {
        if (s >= a.n_slab) break;
        if (!(active >> s & 1)) continue;
        const DSlab& sl = a.slab[s];
        const int l = idx3[sl.axis] - sl.lo;
        if ((unsigned)l >= (unsigned)sl.L) continue;
        const float d1 = sl.axis == 0 ? d[3] : (sl.axis == 1 ? d[5] : d[1]);
        const float d2 = sl.axis == 0 ? d[4] : (sl.axis == 1 ? d[0] : d[2]);
        const float* co = sl.coef + (HSIDE ? 3 * sl.L : 0);
        float p1 = pr.v[s][0], p2 = pr.v[s][1];
        if (!REV) {
            const float ca = FDTD_LDG(co + l), cb = FDTD_LDG(co + sl.L + l);
            p1 = cb * p1 + ca * d1;
            p2 = cb * p2 + ca * d2;
            const long long p = psi_offset(sl, i, j, k);
            a.psi1[s][p] = p1;
            a.psi2[s][p] = p2;
        }
        float c1 = p1, c2 = p2;
        if (!sl.kappa_one) {
            const float ikm1 = FDTD_LDG(co + 2 * sl.L + l) - 1.f;
            c1 = ikm1 * d1 + p1;
            c2 = ikm1 * d2 + p2;
        }
        if (sl.axis == 0) { cu[1] -= c1; cu[2] += c2; }
        else if (sl.axis == 1) { cu[2] -= c1; cu[0] += c2; }
        else { cu[0] -= c1; cu[1] += c2; }
    }
}

// ---------------------------------------------------------------------------------
// The same CPML terms through the per-axis slab table (UpdArgs::axt): the axis of every
// term is a compile-time constant, a cell lies in at most one slab per axis, and a psi
// offset is two 32-bit multiply-adds.  The y and z lookups of a column are fixed along
// the x-march (AxCol); the x lookup is made per plane.
// ---------------------------------------------------------------------------------
template <int AX>
__device__ __forceinline__ int ax_find(const UpdArgs& a, int x, int& l) {
    l = x - a.axs[AX][0].lo;
    if ((unsigned)l < (unsigned)a.axs[AX][0].L) return 0;
    l = x - a.axs[AX][1].lo;
    if ((unsigned)l < (unsigned)a.axs[AX][1].L) return 1;
    return -1;
}

// Offset of (i, j, k) in a slab's psi array for a slab on axis AX (lo, dims sy, sz).
template <int AX>
__device__ __forceinline__ int ax_off(int lo, int sy, int sz, int i, int j, int k) {
    if (AX == 0) return ((i - lo) * sy + j) * sz + k;
    if (AX == 1) return (i * sy + (j - lo)) * sz + k;
    return (i * sy + j) * sz + (k - lo);
}

template <int VEC>
struct AxCol {
    int ys, yl;             // y face of the column (0 / 1, -1: none) and its layer
    int zs[VEC], zl[VEC];   // z face and layer of each of its cells
};

template <int VEC>
__device__ __forceinline__ void ax_column(const UpdArgs& a, int j, int k0, AxCol<VEC>& c) {
    c.ys = ax_find<1>(a, j, c.yl);
#pragma unroll
    for (int e = 0; e < VEC; ++e) c.zs[e] = ax_find<2>(a, k0 + e, c.zl[e]);
}

// Field-wise selection of the slab on face `side` (0 / 1) of axis AX: the table is read
// with static indices only.
#define FDTD_AX_SEL(AX, side, f) ((side) ? a.axs[AX][1].f : a.axs[AX][0].f)
#define FDTD_AX_PSI(AX, side, q) ((side) ? a.axp[AX][1][q] : a.axp[AX][0][q])

// psi pair of the slab on face `side` of axis AX at (i, j, k) (zero when side < 0).
template <int AX>
__device__ __forceinline__ float2 ax_psi(const UpdArgs& a, int side, int i, int j, int k) {
    if (side < 0) return make_float2(0.f, 0.f);
    const int o = ax_off<AX>(FDTD_AX_SEL(AX, side, lo), FDTD_AX_SEL(AX, side, sy), FDTD_AX_SEL(AX, side, sz), i, j, k);
    return make_float2(FDTD_AX_PSI(AX, side, 0)[o], FDTD_AX_PSI(AX, side, 1)[o]);
}

// One slab's CPML term at a cell (cpml_apply for the slab on face `side` of axis AX).
template <bool REV, bool HSIDE, int AX>
__device__ __forceinline__ void ax_term(const UpdArgs& a, int side, int l, int i, int j, int k, const float d[6],
                                        float cu[3], float2 pv) {
    if (side < 0) return;
    const int L = FDTD_AX_SEL(AX, side, L);
    const float d1 = AX == 0 ? d[3] : (AX == 1 ? d[5] : d[1]);
    const float d2 = AX == 0 ? d[4] : (AX == 1 ? d[0] : d[2]);
    const float* co = FDTD_AX_SEL(AX, side, coef) + (HSIDE ? 3 * L : 0);
    float p1 = pv.x, p2 = pv.y;
    if (!REV) {
        const float ca = FDTD_LDG(co + l), cb = FDTD_LDG(co + L + l);
        p1 = cb * p1 + ca * d1;
        p2 = cb * p2 + ca * d2;
        const int o = ax_off<AX>(FDTD_AX_SEL(AX, side, lo), FDTD_AX_SEL(AX, side, sy), FDTD_AX_SEL(AX, side, sz), i, j, k);
        FDTD_AX_PSI(AX, side, 0)[o] = p1;
        FDTD_AX_PSI(AX, side, 1)[o] = p2;
    }
    float c1 = p1, c2 = p2;
    if (!FDTD_AX_SEL(AX, side, kappa_one)) {
        const float ikm1 = FDTD_LDG(co + 2 * L + l) - 1.f;
        c1 = ikm1 * d1 + p1;
        c2 = ikm1 * d2 + p2;
    }
    if (AX == 0) { cu[1] -= c1; cu[2] += c2; }
    else if (AX == 1) { cu[2] -= c1; cu[0] += c2; }
    else { cu[0] -= c1; cu[1] += c2; }
}
#undef FDTD_AX_SEL
#undef FDTD_AX_PSI

// Neighbour on one axis with the halo rule (wrap on a periodic axis, else zero).
__device__ __forceinline__ float nb(const Geo& g, const float* __restrict__ f, long long off, bool inside, int comp, int i,
                                    int j, int k) {
    return inside ? FDTD_LDG(f + off) : ld_halo(g, f, comp, i, j, k);
}

// VEC consecutive z values (16/8/4-byte aligned: nz is a multiple of VEC).
template <int VEC>
struct Vec {
    float v[VEC];
};

template <int VEC>
__device__ __forceinline__ Vec<VEC> ldv(const float* __restrict__ p) {
    Vec<VEC> r;
    if constexpr (VEC == 4) {
        const float4 q = FDTD_LDG(reinterpret_cast<const float4*>(p));
        r.v[0] = q.x; r.v[1] = q.y; r.v[2] = q.z; r.v[3] = q.w;
    } else if constexpr (VEC == 2) {
        const float2 q = FDTD_LDG(reinterpret_cast<const float2*>(p));
        r.v[0] = q.x; r.v[1] = q.y;
    } else {
        r.v[0] = FDTD_LDG(p);
    }
    return r;
}

// Plain (coherent) load of a field this kernel also writes at the same cells.
template <int VEC>
__device__ __forceinline__ Vec<VEC> ldv_rw(const float* p) {
    Vec<VEC> r;
    if constexpr (VEC == 4) {
        const float4 q = FDTD_LDC(reinterpret_cast<const float4*>(p));
        r.v[0] = q.x; r.v[1] = q.y; r.v[2] = q.z; r.v[3] = q.w;
    } else if constexpr (VEC == 2) {
        const float2 q = FDTD_LDC(reinterpret_cast<const float2*>(p));
        r.v[0] = q.x; r.v[1] = q.y;
    } else {
        r.v[0] = FDTD_LDC(p);
    }
    return r;
}

template <int VEC>
__device__ __forceinline__ void stv(float* p, const Vec<VEC>& r) {
    if constexpr (VEC == 4) *reinterpret_cast<float4*>(p) = make_float4(r.v[0], r.v[1], r.v[2], r.v[3]);
    else if constexpr (VEC == 2) *reinterpret_cast<float2*>(p) = make_float2(r.v[0], r.v[1]);
    else *p = r.v[0];
}

template <int VEC>
__device__ __forceinline__ Vec<VEC> ldv_halo(const Geo& g, const float* __restrict__ f, int comp, int i, int j, int k0) {
    Vec<VEC> r;
#pragma unroll
    for (int e = 0; e < VEC; ++e) r.v[e] = ld_halo(g, f, comp, i, j, k0 + e);
    return r;
}

// A neighbour vector one cell away along x or y (all VEC cells share the halo test).
template <int VEC>
__device__ __forceinline__ Vec<VEC> nbv(const Geo& g, const float* __restrict__ f, long long off, bool inside, int comp,
                                        int i, int j, int k0) {
    return inside ? ldv<VEC>(f + off) : ldv_halo<VEC>(g, f, comp, i, j, k0);
}

// The halo loads with the halo rule fixed at compile time: ZH (zero halo, no periodic
// axis) reduces a neighbour outside the grid to a bounds test.
template <bool ZH>
__device__ __forceinline__ float ld_halo_t(const Geo& g, const float* __restrict__ f, int comp, int i, int j, int k) {
    if (!ZH) return ld_halo(g, f, comp, i, j, k);
    const bool in = (unsigned)i < (unsigned)g.nx && (unsigned)j < (unsigned)g.ny && (unsigned)k < (unsigned)g.nz;
    return in ? FDTD_LDG(f + comp * g.N + cell_index(g, i, j, k)) : 0.f;
}

template <bool ZH>
__device__ __forceinline__ float nb_t(const Geo& g, const float* __restrict__ f, long long off, bool inside, int comp,
                                      int i, int j, int k) {
    if (!ZH) return nb(g, f, off, inside, comp, i, j, k);
    return inside ? FDTD_LDG(f + off) : 0.f;
}

template <int VEC, bool ZH>
__device__ __forceinline__ Vec<VEC> ldv_halo_t(const Geo& g, const float* __restrict__ f, int comp, int i, int j, int k0) {
    Vec<VEC> r;
#pragma unroll
    for (int e = 0; e < VEC; ++e) r.v[e] = ld_halo_t<ZH>(g, f, comp, i, j, k0 + e);
    return r;
}

template <int VEC, bool ZH>
__device__ __forceinline__ Vec<VEC> nbv_t(const Geo& g, const float* __restrict__ f, long long off, bool inside, int comp,
                                          int i, int j, int k0) {
    if (!ZH) return nbv<VEC>(g, f, off, inside, comp, i, j, k0);
    if (inside) return ldv<VEC>(f + off);
    Vec<VEC> z;
#pragma unroll
    for (int e = 0; e < VEC; ++e) z.v[e] = 0.f;
    return z;
}

// The slab mask of block `blk`'s box.
template <typename Args>
__device__ __forceinline__ int box_slab_mask_of(const Args& a, int blk) {
    int m = 0;
#pragma unroll
    for (int q = 0; q < 6; ++q)
        if (q < a.nbox && blk >= a.bstart[q]) m = a.bslab[q];
    return m;
}

// Slabs of the box mask that can hold this thread's column: a y or z slab is fixed along the
// x-march (decided once), an x slab is tested per plane (slab_active).
__device__ __forceinline__ int column_slabs(const UpdArgs& a, int box_mask, int j, int k0, int vec) {
    int m = 0;
#pragma unroll
    for (int s = 0; s < FDTD_MAX_SLABS; ++s) {
        if (s >= a.n_slab || !(box_mask >> s & 1)) continue;
        const DSlab& sl = a.slab[s];
        if (sl.axis == 1 && (unsigned)(j - sl.lo) >= (unsigned)sl.L) continue;
        if (sl.axis == 2 && (k0 + vec - 1 < sl.lo || k0 >= sl.lo + sl.L)) continue;
        m |= 1 << s;
    }
    return m;
}

__device__ __forceinline__ int slab_active(const UpdArgs& a, int col_mask, int i) {
    int m = col_mask;
#pragma unroll
    for (int s = 0; s < FDTD_MAX_SLABS; ++s) {
        if (!(col_mask >> s & 1)) continue;
        const DSlab& sl = a.slab[s];
        if (sl.axis == 0 && (unsigned)(i - sl.lo) >= (unsigned)sl.L) m &= ~(1 << s);
    }
    return m;
}

// The material update of one component of one cell.
template <bool REV, bool HSIDE>
__device__ __forceinline__ float material_update(const UpdArgs& a, float u0, float cu, float m, const float* sig_p,
                                                 long long so) {
    const Geo& g = a.g;
    if (sig_p) {
        const float sg = FDTD_LDG(sig_p + so);
        const float q = HSIDE ? g.c * sg / g.eta0 * m / 2.f : g.c * sg * g.eta0 * m / 2.f;
        if (!HSIDE) {
            if (!REV) return ((1.f - q) * u0 + g.c * cu * m) / (1.f + q);
            return (u0 * (1.f + q) - g.c * cu * m) / (1.f - q);
        }
        if (!REV) return ((1.f - q) * u0 - g.c * cu * m) / (1.f + q);
        return (u0 * (1.f + q) + g.c * cu * m) / (1.f - q);
    }
    if (!HSIDE) return REV ? u0 - g.c * cu * m : u0 + g.c * cu * m;
    return REV ? u0 + g.c * cu * m : u0 - g.c * cu * m;
}

// Column decomposition shared by both half-steps: a thread owns VEC consecutive z cells
// of one (j) row and marches over the block's `chunk` x planes.
// The block's box, its column (j, k0) and its x range [i0, i1).  Boxes have VEC-aligned z
// bounds; the box table is indexed with unrolled static indices (no dynamic param access).
template <int VEC, typename Args>
__device__ __forceinline__ bool column_of(const Args& a, int& j, int& k0, int& i0, int& i1, int blk = -1) {
    const int b = blk < 0 ? (int)blockIdx.x : blk;
    int lo0 = 0, lo1 = 0, lo2 = 0, hi0 = 0, hi1 = 0, hi2 = 0, chunk = 1, nbx = 1, start = 0;
#pragma unroll
    for (int q = 0; q < 6; ++q) {
        if (q < a.nbox && b >= a.bstart[q]) {
            lo0 = a.blo[q][0]; lo1 = a.blo[q][1]; lo2 = a.blo[q][2];
            hi0 = a.bhi[q][0]; hi1 = a.bhi[q][1]; hi2 = a.bhi[q][2];
            chunk = a.bchunk[q]; nbx = a.nbx[q]; start = a.bstart[q];
        }
    }
    const int lb = b - start;
    const int by = lb / nbx, bx = lb - by * nbx;
    const int nq = (hi2 - lo2) / VEC;
    // 32-bit column index: a y-z plane holds fewer than 2^31 cells (checked at plan creation)
    const int q = bx * (int)blockDim.x + (int)threadIdx.x;
    if (q >= (hi1 - lo1) * nq) return false;
    const int jj = q / nq;
    j = lo1 + jj;
    k0 = lo2 + (q - jj * nq) * VEC;
    i0 = lo0 + by * chunk;
    i1 = min(i0 + chunk, hi0);
    return i0 < i1;
}

// ---------------------------------------------------------------------------------
// E half-step: E <- (f E + c curl_H(H) inv_eps) / d  (fdtdx/fdtd/update.py:281-354)
// reverse:     E <- (E (1+q) - c curl_H(H) inv_eps) / (1-q)  (update.py:586-609)
// ---------------------------------------------------------------------------------
template <bool REV, int VEC, bool PML, int AXT = 0>
__device__ __forceinline__ void update_E_body(const UpdArgs& a, int blk) {
    constexpr bool ZH = AXT == 2;
    const Geo& g = a.g;
    int j, k0, i0, i1;
    if (!column_of<VEC>(a, j, k0, i0, i1, blk)) return;
    const long long N = g.N;
    const long long sy = g.nz;
    const float* __restrict__ H = a.F;
    const int col = PML && !AXT && a.n_slab > 0 ? column_slabs(a, box_slab_mask_of(a, blk < 0 ? (int)blockIdx.x : blk), j, k0, VEC) : 0;
    AxCol<VEC> axc;
    if (AXT) ax_column<VEC>(a, j, k0, axc);
    Vec<VEC> Hy_m = ldv_halo_t<VEC, ZH>(g, H, 1, i0 - 1, j, k0);
    Vec<VEC> Hz_m = ldv_halo_t<VEC, ZH>(g, H, 2, i0 - 1, j, k0);
    for (int i = i0; i < i1; ++i) {
        const long long c = cell_index(g, i, j, k0);
        const Vec<VEC> Hx = ldv<VEC>(H + c), Hy = ldv<VEC>(H + N + c), Hz = ldv<VEC>(H + 2 * N + c);
        const Vec<VEC> Hz_jm = nbv_t<VEC, ZH>(g, H, 2 * N + c - sy, j > 0, 2, i, j - 1, k0);
        const Vec<VEC> Hx_jm = nbv_t<VEC, ZH>(g, H, c - sy, j > 0, 0, i, j - 1, k0);
        const float Hy_k = nb_t<ZH>(g, H, N + c - 1, k0 > 0, 1, i, j, k0 - 1);   // z neighbour below the vector
        const float Hx_k = nb_t<ZH>(g, H, c - 1, k0 > 0, 0, i, j, k0 - 1);
        Vec<VEC> ie[3];
        if (a.mat) {
#pragma unroll
            for (int comp = 0; comp < 3; ++comp)
                if (comp == 0 || a.n_mat == 3) ie[comp] = ldv<VEC>(a.mat + (a.n_mat == 3 ? comp * N : 0) + c);
            if (a.n_mat != 3) { ie[1] = ie[0]; ie[2] = ie[0]; }
        } else {
#pragma unroll
            for (int comp = 0; comp < 3; ++comp)
#pragma unroll
                for (int e = 0; e < VEC; ++e) ie[comp].v[e] = a.mat_scalar;
        }
        Vec<VEC> Eo[3];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) Eo[comp] = ldv_rw<VEC>(a.Uin + comp * N + c);
        const int act = PML && col ? slab_active(a, col, i) : 0;
        const bool pml = act != 0;
        PsiPre pre[VEC];
        if (pml) {  // issued with the field loads, so both round trips overlap
#pragma unroll
            for (int e = 0; e < VEC; ++e) psi_fetch(a, i, j, k0 + e, pre[e], act);
        }
        int xs = -1, xl = 0;
        float2 px[VEC], py[VEC], pz[VEC];
        if (AXT) {
            xs = ax_find<0>(a, i, xl);
#pragma unroll
            for (int e = 0; e < VEC; ++e) {
                px[e] = ax_psi<0>(a, xs, i, j, k0 + e);
                py[e] = ax_psi<1>(a, axc.ys, i, j, k0 + e);
                pz[e] = ax_psi<2>(a, axc.zs[e], i, j, k0 + e);
            }
        }
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const int k = k0 + e;
            const float hy_km = e == 0 ? Hy_k : Hy.v[e - 1];
            const float hx_km = e == 0 ? Hx_k : Hx.v[e - 1];
            const float d[6] = {Hz.v[e] - Hz_jm.v[e], Hy.v[e] - hy_km, Hx.v[e] - hx_km,
                                Hz.v[e] - Hz_m.v[e], Hy.v[e] - Hy_m.v[e], Hx.v[e] - Hx_jm.v[e]};
            float cu[3] = {d[0] - d[1], d[2] - d[3], d[4] - d[5]};
            if (pml) cpml_apply<REV, false>(a, i, j, k, d, cu, pre[e], act);
            if (AXT) {
                ax_term<REV, false, 0>(a, xs, xl, i, j, k, d, cu, px[e]);
                ax_term<REV, false, 1>(a, axc.ys, axc.yl, i, j, k, d, cu, py[e]);
                ax_term<REV, false, 2>(a, axc.zs[e], axc.zl[e], i, j, k, d, cu, pz[e]);
            }
#pragma unroll
            for (int comp = 0; comp < 3; ++comp) {
                const float* sp = a.sig ? a.sig + (a.n_sig == 3 ? comp * N : 0) : nullptr;
                float u = material_update<REV, false>(a, Eo[comp].v[e], cu[comp], ie[comp].v[e], sp, c + e);
                if (g.pec && face_zero(g, g.pec, comp, i, j, k)) u = 0.f;
                Eo[comp].v[e] = u;
            }
        }
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) stv<VEC>(a.Uout + comp * N + c, Eo[comp]);
        Hy_m = Hy;
        Hz_m = Hz;
    }
}

template <bool REV, int VEC, bool PML, int AXT = 0>
__global__ void __launch_bounds__(256, AXT && VEC == 1 ? 5 : 1) k_update_E(const __grid_constant__ UpdArgs a) {
    update_E_body<REV, VEC, PML, AXT>(a, blockIdx.x);
}

// Accumulates the fused E-only detectors at cell (i, j, k) from the E values the H
// half-step already holds.  Co-location at (i, j, k+1/2) (fdtdx/core/physics/curl.py:120-158):
// Ex <- (avg_x(Ex)(k) + avg_x(Ex)(k+1)) / 2, Ey <- (avg_y(Ey)(k) + avg_y(Ey)(k+1)) / 2, Ez.
// `staged` (optional) points at this cell's previous phasor values of detector 0 in a
// shared-memory tile (complex planes `staged_stride` floats apart), so the read half of
// its read-modify-write comes from the TMA pipeline instead of HBM.  Detectors before `q0`
// are left to the caller.
__device__ __forceinline__ void fused_detectors(const UpdArgs& a, const int slot[kMaxFuse],
                                                const float2 w[kMaxFuse][kMaxFuseFreq], int i, int j, int k,
                                                float Ex, float Ex_kp, float Ex_im, float Exkp_im, float Ey, float Ey_kp,
                                                float Ey_jm, float Eykp_jm, float Ez, const float* staged = nullptr,
                                                int staged_stride = 0, const float2* pref = nullptr, int q0 = 0) {
#pragma unroll
    for (int q = 0; q < kMaxFuse; ++q) {
        if (q < q0) continue;
        if (q >= a.n_fuse) break;
        if (slot[q] < 0) continue;
        const DFuse& d = a.fuse[q];
        if (i < d.lo[0] || i >= d.hi[0] || j < d.lo[1] || j >= d.hi[1] || k < d.lo[2] || k >= d.hi[2]) continue;
        float v[3];
        if (d.exact) {
            v[0] = (0.5f * (Ex + Ex_im) + 0.5f * (Ex_kp + Exkp_im)) / 2.f;
            v[1] = (0.5f * (Ey + Ey_jm) + 0.5f * (Ey_kp + Eykp_jm)) / 2.f;
            v[2] = Ez;
        } else {
            v[0] = Ex;
            v[1] = Ey;
            v[2] = Ez;
        }
        const long long r = ((long long)(i - d.lo[0]) * d.ry + (j - d.lo[1])) * d.rz + (k - d.lo[2]);
        int o = 0;
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            if (!(d.mask >> comp & 1)) continue;
            if (d.kind == FDTD_DET_PHASOR) {
                float2* st = reinterpret_cast<float2*>(d.state);
#pragma unroll
                for (int f = 0; f < kMaxFuseFreq; ++f) {
                    if (f >= d.nfreq) break;
                    float2* pp = st + ((long long)f * d.nout + o) * d.R + r;
                    float2 z;
                    if (q == 0 && staged) {
                        const float* sp = staged + (f * d.nout + o) * staged_stride;
                        z = make_float2(sp[0], sp[1]);
                    } else if (q == 0 && pref) {
                        z = pref[comp];  // prefetched with the field loads (one frequency)
                    } else {
                        z = *pp;
                    }
                    if (d.inverse) { z.x -= v[comp] * w[q][f].x; z.y -= v[comp] * w[q][f].y; }
                    else { z.x += v[comp] * w[q][f].x; z.y += v[comp] * w[q][f].y; }
                    *pp = z;
                }
            } else {
                float* st = reinterpret_cast<float*>(d.state);
                st[((long long)slot[q] * d.nout + o) * d.R + r] = v[comp];
            }
            ++o;
        }
    }
}

// ---------------------------------------------------------------------------------
// H half-step: H <- (g H - c curl_E(E) inv_mu) / e  (fdtdx/fdtd/update.py:717-750)
// reverse:     H <- (H (1+q) + c curl_E(E) inv_mu) / (1-q)  (update.py:905-930)
// Marches along +x keeping E(i+1) (the next iteration's E(i)) and Ex(i-1) in registers;
// fused E-only detectors are accumulated in the same pass (forward only).
// ---------------------------------------------------------------------------------
template <bool REV, int VEC, bool PML, int AXT = 0>
__device__ __forceinline__ void update_H_body(const UpdArgs& a, int blk) {
    constexpr bool ZH = AXT == 2;
    const Geo& g = a.g;
    int j, k0, i0, i1;
    if (!column_of<VEC>(a, j, k0, i0, i1, blk)) return;
    const long long N = g.N;
    const long long sy = g.nz, sx = (long long)g.ny * g.nz;
    const float* __restrict__ E = a.F;
    const bool kin = k0 + VEC < g.nz;
    const int col = PML && !AXT && a.n_slab > 0 ? column_slabs(a, box_slab_mask_of(a, blk < 0 ? (int)blockIdx.x : blk), j, k0, VEC) : 0;
    AxCol<VEC> axc;
    if (AXT) ax_column<VEC>(a, j, k0, axc);

    int slot[kMaxFuse];
    float2 w[kMaxFuse][kMaxFuseFreq];
    bool any = false;
#pragma unroll
    for (int q = 0; q < kMaxFuse; ++q) {
        slot[q] = -1;
        if (REV || q >= a.n_fuse) continue;
        const int t = FDTD_LDC(a.tp);
        slot[q] = FDTD_LDG(a.fuse[q].slot + t + 1);
        any |= slot[q] >= 0;
#pragma unroll
        for (int f = 0; f < kMaxFuseFreq; ++f)
            w[q][f] = (slot[q] >= 0 && f < a.fuse[q].nfreq && a.fuse[q].kind == FDTD_DET_PHASOR)
                          ? FDTD_LDG(a.fuse[q].w + (long long)(t + 1) * a.fuse[q].nfreq + f)
                          : make_float2(0.f, 0.f);
    }

    const long long c0 = cell_index(g, i0, j, k0);
    Vec<VEC> Ey = ldv<VEC>(E + N + c0), Ez = ldv<VEC>(E + 2 * N + c0);
    Vec<VEC> Ex_im{};
    float Exk_im = 0.f;
    if (any) {
        Ex_im = ldv_halo_t<VEC, ZH>(g, E, 0, i0 - 1, j, k0);
        Exk_im = ld_halo_t<ZH>(g, E, 0, i0 - 1, j, k0 + VEC);
    }
    for (int i = i0; i < i1; ++i) {
        const long long c = cell_index(g, i, j, k0);
        const Vec<VEC> Ex = ldv<VEC>(E + c);
        const Vec<VEC> Ey_ip = nbv_t<VEC, ZH>(g, E, N + c + sx, i < g.nx - 1, 1, i + 1, j, k0);
        const Vec<VEC> Ez_ip = nbv_t<VEC, ZH>(g, E, 2 * N + c + sx, i < g.nx - 1, 2, i + 1, j, k0);
        const Vec<VEC> Ez_jp = nbv_t<VEC, ZH>(g, E, 2 * N + c + sy, j < g.ny - 1, 2, i, j + 1, k0);
        const Vec<VEC> Ex_jp = nbv_t<VEC, ZH>(g, E, c + sy, j < g.ny - 1, 0, i, j + 1, k0);
        const float Ey_k = nb_t<ZH>(g, E, N + c + VEC, kin, 1, i, j, k0 + VEC);  // z neighbour above the vector
        const float Ex_k = nb_t<ZH>(g, E, c + VEC, kin, 0, i, j, k0 + VEC);
        Vec<VEC> im[3];
        if (a.mat) {
#pragma unroll
            for (int comp = 0; comp < 3; ++comp)
                if (comp == 0 || a.n_mat == 3) im[comp] = ldv<VEC>(a.mat + (a.n_mat == 3 ? comp * N : 0) + c);
            if (a.n_mat != 3) { im[1] = im[0]; im[2] = im[0]; }
        } else {
#pragma unroll
            for (int comp = 0; comp < 3; ++comp)
#pragma unroll
                for (int e = 0; e < VEC; ++e) im[comp].v[e] = a.mat_scalar;
        }
        Vec<VEC> Ho[3];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) Ho[comp] = ldv_rw<VEC>(a.Uin + comp * N + c);
        const int act = PML && col ? slab_active(a, col, i) : 0;
        const bool pml = act != 0;
        PsiPre pre[VEC];
        if (pml) {
#pragma unroll
            for (int e = 0; e < VEC; ++e) psi_fetch(a, i, j, k0 + e, pre[e], act);
        }
        int xs = -1, xl = 0;
        float2 px[VEC], py[VEC], pz[VEC];
        if (AXT) {
            xs = ax_find<0>(a, i, xl);
#pragma unroll
            for (int e = 0; e < VEC; ++e) {
                px[e] = ax_psi<0>(a, xs, i, j, k0 + e);
                py[e] = ax_psi<1>(a, axc.ys, i, j, k0 + e);
                pz[e] = ax_psi<2>(a, axc.zs[e], i, j, k0 + e);
            }
        }
        Vec<VEC> Ey_jm{};
        float Eyk_jm = 0.f;
        if (!REV && any) {
            Ey_jm = nbv_t<VEC, ZH>(g, E, N + c - sy, j > 0, 1, i, j - 1, k0);
            Eyk_jm = ld_halo_t<ZH>(g, E, 1, i, j - 1, k0 + VEC);
        }
        // the first fused phasor's previous values (one frequency), loaded with the fields so
        // its read-modify-write does not add a second round trip after the update
        // (the per-axis-table kernels also make its update here, from the same region test
        // and index)
        float2 pf[VEC][3];
        bool pfo = false, pin[VEC];
        long long pr[VEC];
        if (!REV && a.n_fuse > 0 && slot[0] >= 0 && a.fuse[0].kind == FDTD_DET_PHASOR && a.fuse[0].nfreq == 1) {
            const DFuse& d = a.fuse[0];
            pfo = true;
            const bool row = i >= d.lo[0] && i < d.hi[0] && j >= d.lo[1] && j < d.hi[1];
            const float2* st = reinterpret_cast<const float2*>(d.state);
#pragma unroll
            for (int e = 0; e < VEC; ++e) {
                const int k = k0 + e;
                const bool in = row && k >= d.lo[2] && k < d.hi[2];
                const long long r = ((long long)(i - d.lo[0]) * d.ry + (j - d.lo[1])) * d.rz + (k - d.lo[2]);
                pin[e] = in;
                pr[e] = r;
                int o = 0;
#pragma unroll
                for (int comp = 0; comp < 3; ++comp) {
                    pf[e][comp] = make_float2(0.f, 0.f);
                    if (!(d.mask >> comp & 1)) continue;
                    if (in) pf[e][comp] = st[(long long)o * d.R + r];
                    ++o;
                }
            }
        }
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const int k = k0 + e;
            const float ey_kp = e + 1 < VEC ? Ey.v[e + 1] : Ey_k;
            const float ex_kp = e + 1 < VEC ? Ex.v[e + 1] : Ex_k;
            const float d[6] = {Ez_jp.v[e] - Ez.v[e], ey_kp - Ey.v[e], ex_kp - Ex.v[e],
                                Ez_ip.v[e] - Ez.v[e], Ey_ip.v[e] - Ey.v[e], Ex_jp.v[e] - Ex.v[e]};
            float cu[3] = {d[0] - d[1], d[2] - d[3], d[4] - d[5]};
            if (pml) cpml_apply<REV, true>(a, i, j, k, d, cu, pre[e], act);
            if (AXT) {
                ax_term<REV, true, 0>(a, xs, xl, i, j, k, d, cu, px[e]);
                ax_term<REV, true, 1>(a, axc.ys, axc.yl, i, j, k, d, cu, py[e]);
                ax_term<REV, true, 2>(a, axc.zs[e], axc.zl[e], i, j, k, d, cu, pz[e]);
            }
#pragma unroll
            for (int comp = 0; comp < 3; ++comp) {
                const float* sp = a.sig ? a.sig + (a.n_sig == 3 ? comp * N : 0) : nullptr;
                float u = material_update<REV, true>(a, Ho[comp].v[e], cu[comp], im[comp].v[e], sp, c + e);
                if (g.pmc && face_zero(g, g.pmc, comp, i, j, k)) u = 0.f;
                Ho[comp].v[e] = u;
            }
            if (!REV && any) {
                const float exkp_im = e + 1 < VEC ? Ex_im.v[e + 1] : Exk_im;
                const float eykp_jm = e + 1 < VEC ? Ey_jm.v[e + 1] : Eyk_jm;
                if (AXT && pfo) {  // the first fused phasor, inline
                    const DFuse& d = a.fuse[0];
                    if (pin[e]) {
                        float v[3];
                        if (d.exact) {
                            v[0] = (0.5f * (Ex.v[e] + Ex_im.v[e]) + 0.5f * (ex_kp + exkp_im)) / 2.f;
                            v[1] = (0.5f * (Ey.v[e] + Ey_jm.v[e]) + 0.5f * (ey_kp + eykp_jm)) / 2.f;
                        } else {
                            v[0] = Ex.v[e];
                            v[1] = Ey.v[e];
                        }
                        v[2] = Ez.v[e];
                        float2* st = reinterpret_cast<float2*>(d.state);
                        const float2 w0 = w[0][0];
                        int o = 0;
#pragma unroll
                        for (int comp = 0; comp < 3; ++comp) {
                            if (!(d.mask >> comp & 1)) continue;
                            float2 z = pf[e][comp];
                            if (d.inverse) { z.x -= v[comp] * w0.x; z.y -= v[comp] * w0.y; }
                            else { z.x += v[comp] * w0.x; z.y += v[comp] * w0.y; }
                            st[(long long)o * d.R + pr[e]] = z;
                            ++o;
                        }
                    }
                    if (a.n_fuse > 1)
                        fused_detectors(a, slot, w, i, j, k, Ex.v[e], ex_kp, Ex_im.v[e], exkp_im, Ey.v[e], ey_kp,
                                        Ey_jm.v[e], eykp_jm, Ez.v[e], nullptr, 0, nullptr, 1);
                } else {
                    fused_detectors(a, slot, w, i, j, k, Ex.v[e], ex_kp, Ex_im.v[e], exkp_im, Ey.v[e], ey_kp, Ey_jm.v[e],
                                    eykp_jm, Ez.v[e], nullptr, 0, pfo ? pf[e] : nullptr);
                }
            }
        }
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) stv<VEC>(a.Uout + comp * N + c, Ho[comp]);
        Ex_im = Ex;
        Exk_im = Ex_k;
        Ey = Ey_ip;
        Ez = Ez_ip;
    }
}

template <bool REV, int VEC, bool PML, int AXT = 0>
__global__ void __launch_bounds__(256, AXT && VEC == 1 ? (REV ? 5 : 4) : 3) k_update_H(const __grid_constant__ UpdArgs a) {
    update_H_body<REV, VEC, PML, AXT>(a, blockIdx.x);
}

// ---------------------------------------------------------------------------------
// Source injection.  One thread per source cell.  `inverse` flips the sign (the
// reverse step subtracts what the forward step added).  Positions a conductor
// wall zeroes are skipped: the wall's zeroing runs after the injection in the
// reference, so an injection there never survives.
// Point dipole: fdtdx/objects/sources/dipole.py:195-277.
// TFSF plane:   fdtdx/objects/sources/tfsf.py:193-409, 739-806.
// ---------------------------------------------------------------------------------
__device__ __forceinline__ float mat_at(const float* m, int n, float scalar, long long N, int comp, long long c) {
    if (!m) return scalar;
    // an isotropic array serves every component; a full tensor's diagonal entry is comp * 4
    const int cc = n == 9 ? comp * 4 : (comp < n ? comp : n - 1);
    return FDTD_LDG(m + cc * N + c);
}

template <bool ESIDE>
__device__ __forceinline__ void source_body(const Geo& g, const DSource& s, const int* __restrict__ tp, float* F,
                                            const float* mat, int n_mat, float mat_scalar, int inverse, int blk) {
    const int wall = ESIDE ? g.pec : g.pmc;
    if (s.kind == FDTD_SRC_DIPOLE) {
        if (blk != 0 || threadIdx.x != 0) return;
        if (ESIDE == (bool)s.magnetic) return;
        const int i = s.lo[0], j = s.lo[1], k = s.lo[2];
        if (face_zero(g, wall, s.comp, i, j, k)) return;
        const int ti = FDTD_LDC(tp) + 1;
        if (!s.on[ti]) return;
        const float amp = profile_amp(s, s.teff[ti] + (ESIDE ? 0.f : 0.5f), ESIDE ? s.phE[ti] : s.phH[ti]);
        const float sg = inverse ? 1.f : -1.f;
        atomicAdd(F + s.comp * g.N + cell_index(g, i, j, k), sg * (s.coef * amp));
        return;
    }
    const int n = s.normal, ax = (n + 1) % 3, bx = (n + 2) % 3;
    const int ext[3] = {s.hi[0] - s.lo[0], s.hi[1] - s.lo[1], s.hi[2] - s.lo[2]};
    const long long P = (long long)ext[0] * ext[1] * ext[2];
    const long long f = (long long)blk * blockDim.x + threadIdx.x;
    if (f >= P) return;
    const int kk = (int)(f % ext[2]);
    const int jj = (int)((f / ext[2]) % ext[1]);
    const int ii = (int)(f / ((long long)ext[2] * ext[1]));
    const int i = s.lo[0] + ii, j = s.lo[1] + jj, k = s.lo[2] + kk;
    const long long c = cell_index(g, i, j, k);
    const float sg = inverse ? -s.sign : s.sign;
    const float* inc = ESIDE ? s.incH : s.incE;
    const float* off = ESIDE ? s.offH : s.offE;
    // every load that does not depend on the time step is issued before the step counter's,
    // and the field is updated by atomic adds (no read of it; sources that overlap, which a
    // batched launch runs together, add up in any order), so the kernel waits on two memory
    // round trips instead of five
    const float oa = FDTD_LDG(off + ax * P + f), ob = FDTD_LDG(off + bx * P + f);
    const float ia = FDTD_LDG(inc + ax * P + f), ib = FDTD_LDG(inc + bx * P + f);
    const float ma = mat_at(mat, n_mat, mat_scalar, g.N, ax, c), mb = mat_at(mat, n_mat, mat_scalar, g.N, bx, c);
    const int ti = FDTD_LDC(tp) + 1;
    if (!s.on[ti]) return;
    const float teff = s.teff[ti] + (ESIDE ? 0.f : 0.5f);
    const float ph0 = ESIDE ? s.phE[ti] : s.phH[ti];
    // E side in a dispersive scene: the broadband-filtered table of the H incident profile
    const bool tab = ESIDE && s.etab;
    const float amp_a = tab ? table_amp(s, teff + oa) : profile_amp(s, teff + oa, ph0 + s.omega_dt * oa);
    const float amp_b = tab ? table_amp(s, teff + ob) : profile_amp(s, teff + ob, ph0 + s.omega_dt * ob);
    const float inc_a = ia * amp_a;
    const float inc_b = ib * amp_b;
    if (mat && n_mat == 9) {
        // a full tensor on the face (tfsf.py:287-299, 384-393): every row takes both tangential
        // terms through its (row, a) and (row, b) entries
        const int rows[3] = {n, ax, bx};
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            const int row = rows[q];
            if (face_zero(g, wall, row, i, j, k)) continue;
            const float mra = FDTD_LDG(mat + (row * 3 + ax) * g.N + c), mrb = FDTD_LDG(mat + (row * 3 + bx) * g.N + c);
            const float corr = ESIDE ? mra * inc_b - mrb * inc_a : mrb * inc_a - mra * inc_b;
            atomicAdd(F + row * g.N + c, sg * (s.coef * corr));
        }
        return;
    }
    if (ESIDE) {
        // E[a] += sign c inv_eps[a] H_inc,b ;  E[b] -= sign c inv_eps[b] H_inc,a
        if (!face_zero(g, wall, ax, i, j, k)) atomicAdd(F + ax * g.N + c, sg * (inc_b * s.coef * ma));
        if (!face_zero(g, wall, bx, i, j, k)) atomicAdd(F + bx * g.N + c, -(sg * (inc_a * s.coef * mb)));
    } else {
        // H[b] += sign c inv_mu[b] E_inc,a ;  H[a] -= sign c inv_mu[a] E_inc,b
        if (!face_zero(g, wall, bx, i, j, k)) atomicAdd(F + bx * g.N + c, sg * (inc_a * s.coef * mb));
        if (!face_zero(g, wall, ax, i, j, k)) atomicAdd(F + ax * g.N + c, -(sg * (inc_b * s.coef * ma)));
    }
}

// ADE polarisation step before the E update (fdtdx/fdtd/update.py:316-350), one thread per
// component and cell: P_hat = c1 P^n + c2 P^(n-1) + c3 E^n for every pole, P^(n-1) <- P^n,
// P^n <- P_hat, and E^n <- E^n + inv_eps sum_poles (P^n - P_hat) / f with f = 1 - q the
// conductivity factor, so that the E kernel's (f E + c curl inv_eps) / (1 + q) equals the
// reference's (f E + c curl inv_eps + inv_eps sum (P^n - P_hat)) / (1 + q).  Cells without a
// pole hold zero coefficients and stay unchanged.
__global__ void __launch_bounds__(256) k_ade(const Geo g, float* __restrict__ E, float* __restrict__ Pc,
                                             float* __restrict__ Pp, const float* __restrict__ c1,
                                             const float* __restrict__ c2, const float* __restrict__ c3, int np, int nd,
                                             const float* __restrict__ inv_eps, int n_eps, const float* __restrict__ sig,
                                             int n_sig) {
    const long long N = g.N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3 * N) return;
    const int comp = (int)(idx / N);
    const long long c = idx - comp * N;
    const float e = E[idx];
    float delta = 0.f;
    for (int p = 0; p < np; ++p) {
        const long long pi = ((long long)p * 3 + comp) * N + c;
        const long long ci = ((long long)p * nd + (nd == 3 ? comp : 0)) * N + c;
        const float pc = Pc[pi], pp = Pp[pi];
        const float ph = FDTD_LDG(c1 + ci) * pc + FDTD_LDG(c2 + ci) * pp + FDTD_LDG(c3 + ci) * e;
        delta += pc - ph;
        Pp[pi] = pc;
        Pc[pi] = ph;
    }
    const float m = FDTD_LDG(inv_eps + (n_eps == 3 ? comp : 0) * N + c);
    float add = m * delta;
    if (sig) add /= 1.f - g.c * FDTD_LDG(sig + (n_sig == 3 ? comp : 0) * N + c) * g.eta0 * m / 2.f;
    E[idx] = e + add;
}

template <bool ESIDE>
__global__ void k_source(const Geo g, const DSource s, const int* __restrict__ tp, float* F, const float* mat, int n_mat,
                         float mat_scalar, int inverse) {
    source_body<ESIDE>(g, s, tp, F, mat, n_mat, mat_scalar, inverse, blockIdx.x);
}

// ---------------------------------------------------------------------------------
// Detectors (fdtdx/fdtd/update.py:1040-1137).  Fields are co-located at the E_z
// point (i, j, k+1/2) with H time-centred as (H_prev + H)/2 when
// exact_interpolation is set (fdtdx/core/physics/curl.py:86-224).
// ---------------------------------------------------------------------------------
struct DetFields {
    const float* E;
    const float* Hp;   // H before this step's H update
    const float* H;    // H after it
    const float* inv_eps;
    int n_eps;
    const float* inv_mu;
    int n_mu;
    float mu_scalar;
    long long im = 0;  // complex (Bloch) fields: floats from each field's real parts to its imaginary parts
};

__device__ __forceinline__ float hav(const Geo& g, const DetFields& f, int comp, int i, int j, int k) {
    return (ld_halo_sel(g, f.Hp, comp, i, j, k) + ld_halo_sel(g, f.H, comp, i, j, k)) / 2.f;
}

__device__ void colocate(const Geo& g, const DetFields& f, int exact, int mask, int i, int j, int k, float v[6]) {
    const long long c = cell_index(g, i, j, k);
    if (!exact) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            v[q] = (mask >> q & 1) ? FDTD_LDG(f.E + q * g.N + c) : 0.f;
            v[3 + q] = (mask >> (3 + q) & 1) ? FDTD_LDG(f.H + q * g.N + c) : 0.f;
        }
        return;
    }
    if (mask & 1) {
        const float lo = 0.5f * (ld_halo_sel(g, f.E, 0, i, j, k) + ld_halo_sel(g, f.E, 0, i - 1, j, k));
        const float up = 0.5f * (ld_halo_sel(g, f.E, 0, i, j, k + 1) + ld_halo_sel(g, f.E, 0, i - 1, j, k + 1));
        v[0] = (lo + up) / 2.f;
    }
    if (mask & 2) {
        const float lo = 0.5f * (ld_halo_sel(g, f.E, 1, i, j, k) + ld_halo_sel(g, f.E, 1, i, j - 1, k));
        const float up = 0.5f * (ld_halo_sel(g, f.E, 1, i, j, k + 1) + ld_halo_sel(g, f.E, 1, i, j - 1, k + 1));
        v[1] = (lo + up) / 2.f;
    }
    if (mask & 4) v[2] = FDTD_LDG(f.E + 2 * g.N + c);
    if (mask & 8) v[3] = 0.5f * (hav(g, f, 0, i, j, k) + hav(g, f, 0, i, j - 1, k));
    if (mask & 16) v[4] = 0.5f * (hav(g, f, 1, i, j, k) + hav(g, f, 1, i - 1, j, k));
    if (mask & 32) {
        const float lx = 0.5f * (hav(g, f, 2, i, j, k) + hav(g, f, 2, i - 1, j, k));
        const float lxy = 0.5f * (lx + 0.5f * (hav(g, f, 2, i, j - 1, k) + hav(g, f, 2, i - 1, j - 1, k)));
        const float ux = 0.5f * (hav(g, f, 2, i, j, k + 1) + hav(g, f, 2, i - 1, j, k + 1));
        const float uxy = 0.5f * (ux + 0.5f * (hav(g, f, 2, i, j - 1, k + 1) + hav(g, f, 2, i - 1, j - 1, k + 1)));
        v[5] = (lxy + uxy) / 2.f;
    }
}

template <int BLOCK>
__device__ __forceinline__ float block_sum(float x, float* sh) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    __syncthreads();
    if (lane == 0) sh[w] = x;
    __syncthreads();
    float r = 0.f;
    if (w == 0) {
        r = lane < BLOCK / 32 ? sh[lane] : 0.f;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) r += __shfl_down_sync(0xffffffffu, r, o);
    }
    return r;  // valid in thread 0
}

constexpr int kDetBlock = 256;

__device__ __forceinline__ void detector_body(const Geo& g, const DDet& d, const int* __restrict__ tp,
                                              const DetFields& f, void* state, int blk) {
    __shared__ float sh[kDetBlock / 32];
    const long long r = (long long)blk * blockDim.x + threadIdx.x;
    const bool valid = r < d.R;
    float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    int i = 0, j = 0, k = 0;
    if (valid) {
        k = d.lo[2] + (int)(r % d.rz);
        j = d.lo[1] + (int)((r / d.rz) % d.ry);
        i = d.lo[0] + (int)(r / ((long long)d.rz * d.ry));
    }
    int need = d.comp_mask;
    if (d.kind == FDTD_DET_FLUX || d.kind == FDTD_DET_ENERGY) need = 63;
    // complex (Bloch) fields: the imaginary parts' samples too, with the other part and sign
    // of each wrapped neighbour's phase mixing swapped
    float vi[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    // the samples do not depend on the step: their loads are issued before the step
    // counter's and the slot table's, which then overlap them
    if (valid) {
        colocate(g, f, d.exact, need, i, j, k, v);
        if (f.im && d.kind != FDTD_DET_FIELD) {
            Geo gi = g;
            gi.pother = -f.im;
            gi.psign = 1.f;
            DetFields fi = f;
            fi.E = f.E + f.im;
            fi.Hp = f.Hp + f.im;
            fi.H = f.H + f.im;
            colocate(gi, fi, d.exact, need, i, j, k, vi);
        }
    }
    const int t = FDTD_LDC(tp);
    const int slot = FDTD_LDG(d.slot + t + 1);
    if (slot < 0) return;

    // gather the recorded values of this cell (outi: the imaginary parts of complex phasor
    // samples; a field detector of complex fields records their real parts)
    float out[6], outi[6];
    int nout = 0;
    if (d.kind == FDTD_DET_FIELD || d.kind == FDTD_DET_PHASOR) {
#pragma unroll
        for (int q = 0; q < 6; ++q)
            if (d.comp_mask >> q & 1) {
                outi[nout] = vi[q];
                out[nout++] = v[q];
            }
    } else if (d.kind == FDTD_DET_FLUX) {
        // S = E x H (real fields; fdtdx/core/physics/metrics.py:99-117); complex fields:
        // Re(E x conj H) = E_re x H_re + E_im x H_im
        float S[3] = {v[1] * v[5] - v[2] * v[4], v[2] * v[3] - v[0] * v[5], v[0] * v[4] - v[1] * v[3]};
        if (f.im) {
            S[0] += vi[1] * vi[5] - vi[2] * vi[4];
            S[1] += vi[2] * vi[3] - vi[0] * vi[5];
            S[2] += vi[0] * vi[4] - vi[1] * vi[3];
        }
        if (d.keep_all) {
            out[0] = d.flux_sign * S[0];
            out[1] = d.flux_sign * S[1];
            out[2] = d.flux_sign * S[2];
            nout = 3;
        } else {
            out[0] = d.flux_sign * S[d.flux_axis];
            nout = 1;
        }
    } else {  // energy: 0.5 sum eps |E|^2 + 0.5 sum mu |H|^2 (fdtdx/core/physics/metrics.py:55-65)
        float e = 0.f, h = 0.f;
        if (valid && (f.n_eps == 9 || (f.inv_mu && f.n_mu == 9))) {
            // full tensors: 0.5 Re(E* eps E) + 0.5 Re(H* mu H), eps and mu the inverses of the
            // stored inverse tensors (metrics.py:34-51)
            const long long c = cell_index(g, i, j, k);
            float t[9], m[9];
            tensor_at(f.inv_eps, f.n_eps, 1.f, g.N, c, t);
            inverse3(t, m);
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int q = 0; q < 3; ++q) e += 0.5f * m[p * 3 + q] * (v[p] * v[q] + vi[p] * vi[q]);
            tensor_at(f.inv_mu, f.n_mu, f.mu_scalar, g.N, c, t);
            inverse3(t, m);
#pragma unroll
            for (int p = 0; p < 3; ++p)
#pragma unroll
                for (int q = 0; q < 3; ++q) h += 0.5f * m[p * 3 + q] * (v[3 + p] * v[3 + q] + vi[3 + p] * vi[3 + q]);
        } else if (valid) {
            const long long c = cell_index(g, i, j, k);
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                e += 0.5f * (1.f / mat_at(f.inv_eps, f.n_eps, 1.f, g.N, q, c)) * (v[q] * v[q] + vi[q] * vi[q]);
                h += 0.5f * (1.f / mat_at(f.inv_mu, f.n_mu, f.mu_scalar, g.N, q, c)) *
                     (v[3 + q] * v[3 + q] + vi[3 + q] * vi[3 + q]);
            }
        }
        out[0] = e + h;
        nout = 1;
    }

    if (d.kind == FDTD_DET_PHASOR) {
        const float2* wt = d.w + (long long)(t + 1) * d.nfreq;
        if (!d.reduce) {
            if (!valid) return;
            float2* st = reinterpret_cast<float2*>(state);
            for (int fq = 0; fq < d.nfreq; ++fq) {
                const float2 w = FDTD_LDG(wt + fq);
                for (int q = 0; q < nout; ++q) {
                    float2* p = st + ((long long)fq * nout + q) * d.R + r;
                    float2 z = *p;
                    // the sample (out + i outi) times the weight
                    const float ar = f.im ? out[q] * w.x - outi[q] * w.y : out[q] * w.x;
                    const float ai = f.im ? out[q] * w.y + outi[q] * w.x : out[q] * w.y;
                    if (d.inverse) { z.x -= ar; z.y -= ai; }
                    else { z.x += ar; z.y += ai; }
                    *p = z;
                }
            }
            return;
        }
        // volume mean of the complex samples: partials (2 floats per freq and component)
        for (int fq = 0; fq < d.nfreq; ++fq) {
            const float2 w = FDTD_LDG(wt + fq);
            for (int q = 0; q < nout; ++q) {
                const float ar = f.im ? out[q] * w.x - outi[q] * w.y : out[q] * w.x;
                const float ai = f.im ? out[q] * w.y + outi[q] * w.x : out[q] * w.y;
                const float re = block_sum<kDetBlock>(valid ? ar : 0.f, sh);
                const float im = block_sum<kDetBlock>(valid ? ai : 0.f, sh);
                if (threadIdx.x == 0) {
                    d.partial[(long long)blk * d.ncomp + 2 * (fq * nout + q)] = re;
                    d.partial[(long long)blk * d.ncomp + 2 * (fq * nout + q) + 1] = im;
                }
            }
        }
        return;
    }
    if (!d.reduce) {
        if (!valid) return;
        float* st = reinterpret_cast<float*>(state);
        for (int q = 0; q < nout; ++q) st[((long long)slot * nout + q) * d.R + r] = out[q];
        return;
    }
    for (int q = 0; q < nout; ++q) {
        const float s = block_sum<kDetBlock>(valid ? out[q] : 0.f, sh);
        if (threadIdx.x == 0) d.partial[(long long)blk * d.ncomp + q] = s;
    }
}

__global__ void __launch_bounds__(kDetBlock) k_detector(const Geo g, const DDet d, const int* __restrict__ tp,
                                                        const DetFields f, void* state) {
    detector_body(g, d, tp, f, state, blockIdx.x);
}

// Sums the block partials of a reducing detector in a fixed order (deterministic)
// and writes (field, flux, energy) or accumulates (phasor) the state entry.
__device__ __forceinline__ void detector_finalize_body(const DDet& d, const int* __restrict__ tp, void* state) {
    __shared__ float sh[kDetBlock / 32];
    const int t = FDTD_LDC(tp);
    const int slot = FDTD_LDG(d.slot + t + 1);
    if (slot < 0) return;
    for (int q = 0; q < d.ncomp; ++q) {
        float acc = 0.f;
        for (int b = threadIdx.x; b < d.nblocks; b += blockDim.x) acc += FDTD_LDC(d.partial + (long long)b * d.ncomp + q);
        const float s = block_sum<kDetBlock>(acc, sh);
        if (threadIdx.x == 0) {
            if (d.kind == FDTD_DET_PHASOR) {
                float* st = reinterpret_cast<float*>(state);
                const float v = s / (float)d.R;
                st[q] += d.inverse ? -v : v;
            } else {
                float* st = reinterpret_cast<float*>(state);
                const float scale = d.kind == FDTD_DET_FIELD ? 1.f / (float)d.R : d.cell_weight;
                st[(long long)slot * d.ncomp + q] = s * scale;
            }
        }
    }
}

__global__ void __launch_bounds__(kDetBlock) k_detector_finalize(const DDet d, const int* __restrict__ tp, void* state) {
    detector_finalize_body(d, tp, state);
}

// ---------------------------------------------------------------------------------
// PML-interface recording (fdtdx/fdtd/misc.py:10-66, fdtdx/fdtd/update.py:1140-1222):
// E and H on the innermost layer of every slab.  Slot layout: for field in (E, H):
// for slab s: (3, plane_s).  RESTORE copies the slot back into the fields.
// ---------------------------------------------------------------------------------
struct IfaceDev {
    int n;
    int axis[FDTD_MAX_SLABS];
    int layer[FDTD_MAX_SLABS];
    long long start[FDTD_MAX_SLABS + 1];  // prefix sums of plane sizes
    long long total;                     // sum of plane sizes
    // recorder time filter (nullptr: one slot per step): store slot, restore slots a, b, weight
    const int* store;
    const int* ra;
    const int* rb;
    const float* rw;
};

template <typename T, bool RESTORE>
__device__ __forceinline__ void interfaces_body(const Geo& g, const IfaceDev& ifc, const int* __restrict__ tp,
                                                int n_slots, float* E, float* H, T* rec, int blk) {
    const long long q = (long long)blk * blockDim.x + threadIdx.x;
    if (q >= ifc.total) return;
    int s = 0;
    while (s + 1 < ifc.n && q >= ifc.start[s + 1]) ++s;
    const long long pidx = q - ifc.start[s];
    int i, j, k;
    if (ifc.axis[s] == 0) { i = ifc.layer[s]; j = (int)(pidx / g.nz); k = (int)(pidx % g.nz); }
    else if (ifc.axis[s] == 1) { j = ifc.layer[s]; i = (int)(pidx / g.nz); k = (int)(pidx % g.nz); }
    else { k = ifc.layer[s]; i = (int)(pidx / g.ny); j = (int)(pidx % g.ny); }
    const long long c = cell_index(g, i, j, k);
    // recording: the field values do not depend on the step, so they are loaded before the
    // step counter and its table (one memory round trip less on the critical path)
    float v[6];
    if (!RESTORE) {
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            v[comp] = FDTD_LDC(E + comp * g.N + c);
            v[3 + comp] = FDTD_LDC(H + comp * g.N + c);
        }
    }
    int t = FDTD_LDC(tp), tb = t;
    float w = 0.f;
    if (ifc.store) {  // time filter: store every k-th step, restore by linear interpolation
        const int ti = t + 1;
        if (RESTORE) {
            tb = FDTD_LDG(ifc.rb + ti);
            w = FDTD_LDG(ifc.rw + ti);
            t = FDTD_LDG(ifc.ra + ti);
        } else {
            t = tb = FDTD_LDG(ifc.store + ti);
            if (t < 0) return;
        }
    } else {
        if (t < 0) t += n_slots;  // a negative step index wraps like a JAX index
        tb = t;
    }
    if (t < 0 || t >= n_slots || tb < 0 || tb >= n_slots) return;
    const long long P = ifc.start[s + 1] - ifc.start[s];
    T* slotp = rec + (long long)t * 6 * ifc.total;
    const long long db = ((long long)tb - t) * 6 * ifc.total;  // slot b relative to slot a
#pragma unroll
    for (int fld = 0; fld < 2; ++fld) {
        T* base = slotp + fld * 3 * ifc.total + 3 * ifc.start[s];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            if (RESTORE) {
                float* F = fld == 0 ? E : H;
                const float va = from_storage(base[comp * P + pidx]);
                F[comp * g.N + c] = w != 0.f ? va + w * (from_storage(base[db + comp * P + pidx]) - va) : va;
            } else {
                base[comp * P + pidx] = to_storage<T>(v[3 * fld + comp]);
            }
        }
    }
}

template <typename T, bool RESTORE>
__global__ void k_interfaces(const Geo g, const IfaceDev ifc, const int* __restrict__ tp, int n_slots, float* E, float* H,
                             T* rec) {
    interfaces_body<T, RESTORE>(g, ifc, tp, n_slots, E, H, rec, blockIdx.x);
}

__global__ void k_set_step(int* tp, int t) { *tp = t; }
__global__ void k_advance(int* tp, int delta) { *tp += delta; }

// Sets *err to FDTD_ENONFINITE when any of the n floats at f is a NaN or an infinity
// (grid-stride, one flag per block).  Reads only; the fields are left as they are.
__global__ void __launch_bounds__(256) k_check_finite(const float* __restrict__ f, long long n, int* err) {
    bool bad = false;
    const long long stride = (long long)gridDim.x * blockDim.x;
    for (long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x; q < n; q += stride)
        bad |= !isfinite(FDTD_LDG(f + q));
    if (__syncthreads_or(bad) && threadIdx.x == 0) atomicExch(err, FDTD_ENONFINITE);
}

}  // namespace fdtd
