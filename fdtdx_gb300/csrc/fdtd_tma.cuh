// TMA-pipelined Yee half-steps (sm_103a).
//
// A block owns a TY x TZ tile of (y, z) columns and marches over `chunk` x planes.
// For every plane one elected thread issues cp.async.bulk.tensor loads of the
// plane's tiles into a shared-memory stage (the differentiated field with a one-cell
// halo, the updated field, the material and the conductivity), completing on the
// stage's mbarrier; NS stages are in flight, so the data waiting on HBM lives in
// shared memory instead of registers.  Out-of-range tile cells read as zero (TMA
// fill), which is exactly the reference's zero halo (fdtdx/core/misc.py:615-641);
// scenes with a periodic axis use the register-queue kernels instead.  These kernels
// update the core box of the grid, which holds no CPML cell; the slabs are updated by
// the register-queue kernels with their CPML corrections.
//
// Every mbarrier wait is bounded: a wait that runs out sets the plan's error word to
// FDTD_ETIMEOUT, the block learns it through __syncthreads_or, the elected thread waits
// (bounded) for the copies it issued and the block returns.
#pragma once

#include <cuda.h>

#include "fdtd_kernels.cuh"

namespace fdtd {

constexpr uint32_t kWaitLimit = 1u << 22;
constexpr int kMaxStages = 6;

struct TmaCfg {
    int TZ, TY, ns;
    int nm, nsig;          // components of the material / conductivity tiles (0: none)
    int nd;                // complex planes (freqs x components) of the staged detector tile (0: none)
    int dlo[3];            // region origin of the staged detector
    int off_U, off_M, off_S, off_D, stage_floats;
    uint32_t stage_bytes;  // bytes the TMA loads of one stage deliver
    int* err;
    int expire;            // test hook: take the bounded-wait error exit before issuing any copy
};

// ---------------------------------------------------------------------------------
// CPML terms inside the TMA half-steps (PML kernels: a box that may hold slab cells, up to
// the whole grid).  The layer of a thread's column in a y or z slab is fixed along the whole
// x-march (YCol, ZCol: coefficients read once, the psi offset grows by a constant per plane);
// the x layer is the same for every thread of a plane (XPlane, block-uniform loads).  psi is
// read a plane ahead of its use (PsiPf) with plain loads, one 8-byte access per psi array for
// a thread's two cells.  The terms are those of ax_term (fdtdx/core/physics/curl.py:284-308,
// perfectly_matched_layer.py:138-190), applied in axis order x, y, z as the shell kernel
// applies them.  psi offsets: x slab (L, ny, nz) -> (l ny + j) nz + k; y slab (nx, L, nz) ->
// (i L + l) nz + k; z slab (nx, ny, L) -> (i ny + j) L + l.
// ---------------------------------------------------------------------------------
struct ZCol {
    int o[2];              // psi offset of each cell at plane 0 (-1: the cell has no z term)
    int stride;            // psi floats per x plane (ny L)
    float ca[2], cb[2], km[2];
    int kone;
    float* p1;
    float* p2;
};

template <bool HSIDE>
__device__ __forceinline__ void zcol_init(const UpdArgs& a, int j, int k0, bool valid, ZCol& z) {
    z.o[0] = z.o[1] = -1;
    z.stride = 0;
    z.kone = 1;
    z.p1 = z.p2 = nullptr;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        z.ca[e] = z.cb[e] = z.km[e] = 0.f;
        int l = 0;
        const int side = valid ? ax_find<2>(a, k0 + e, l) : -1;
        if (side < 0) continue;
        // two adjacent cells cannot lie in the two different z slabs: one side per thread
        const int L = side ? a.axs[2][1].L : a.axs[2][0].L;
        const float* co = (side ? a.axs[2][1].coef : a.axs[2][0].coef) + (HSIDE ? 3 * L : 0);
        z.kone = side ? a.axs[2][1].kappa_one : a.axs[2][0].kappa_one;
        z.p1 = side ? a.axp[2][1][0] : a.axp[2][0][0];
        z.p2 = side ? a.axp[2][1][1] : a.axp[2][0][1];
        z.stride = a.g.ny * L;
        z.o[e] = j * L + l;
        z.ca[e] = __ldg(co + l);
        z.cb[e] = __ldg(co + L + l);
        z.km[e] = z.kone ? 0.f : __ldg(co + 2 * L + l) - 1.f;
    }
}

struct YCol {
    int o[2];              // psi offset of each cell at plane 0 (-1: no y term)
    int stride;            // psi floats per x plane (L nz)
    float ca, cb, km;
    int kone;
    float* p1;
    float* p2;
};

template <bool HSIDE>
__device__ __forceinline__ void ycol_init(const UpdArgs& a, int j, int k0, bool valid, YCol& y) {
    y.o[0] = y.o[1] = -1;
    y.ca = y.cb = y.km = 0.f;
    y.kone = 1;
    y.stride = 0;
    y.p1 = y.p2 = nullptr;
    int l = 0;
    const int side = ax_find<1>(a, j, l);
    if (!valid || side < 0) return;
    const int L = side ? a.axs[1][1].L : a.axs[1][0].L;
    const float* co = (side ? a.axs[1][1].coef : a.axs[1][0].coef) + (HSIDE ? 3 * L : 0);
    y.kone = side ? a.axs[1][1].kappa_one : a.axs[1][0].kappa_one;
    y.p1 = side ? a.axp[1][1][0] : a.axp[1][0][0];
    y.p2 = side ? a.axp[1][1][1] : a.axp[1][0][1];
    y.ca = __ldg(co + l);
    y.cb = __ldg(co + L + l);
    y.km = y.kone ? 0.f : __ldg(co + 2 * L + l) - 1.f;
    y.stride = L * a.g.nz;
    y.o[0] = l * a.g.nz + k0;
    y.o[1] = y.o[0] + 1;
}

struct XPlane {
    int side, l;           // face of the x slab holding the plane (-1: none) and its layer
    float ca, cb, km;
    int kone;
    float* p1;
    float* p2;
};

template <bool HSIDE>
__device__ __forceinline__ void xplane_init(const UpdArgs& a, int i, XPlane& x) {
    x.side = ax_find<0>(a, i, x.l);
    x.ca = x.cb = x.km = 0.f;
    x.kone = 1;
    x.p1 = x.p2 = nullptr;
    if (x.side < 0) return;
    const int L = x.side ? a.axs[0][1].L : a.axs[0][0].L;
    const float* co = (x.side ? a.axs[0][1].coef : a.axs[0][0].coef) + (HSIDE ? 3 * L : 0);
    x.kone = x.side ? a.axs[0][1].kappa_one : a.axs[0][0].kappa_one;
    x.p1 = x.side ? a.axp[0][1][0] : a.axp[0][0][0];
    x.p2 = x.side ? a.axp[0][1][1] : a.axp[0][0][1];
    x.ca = __ldg(co + x.l);
    x.cb = __ldg(co + L + x.l);
    x.km = x.kone ? 0.f : __ldg(co + 2 * L + x.l) - 1.f;
}

__device__ __forceinline__ int xplane_off(const UpdArgs& a, const XPlane& x, int j, int k) {
    return (x.l * a.g.ny + j) * a.g.nz + k;
}

// psi offsets of a thread's two cells at plane i (-1: no term there).
__device__ __forceinline__ void zcol_off(const ZCol& z, int i, int& o0, int& o1) {
    o0 = z.o[0] >= 0 ? z.o[0] + i * z.stride : -1;
    o1 = z.o[1] >= 0 ? z.o[1] + i * z.stride : -1;
}

__device__ __forceinline__ void ycol_off(const YCol& y, int i, int& o0, int& o1) {
    o0 = y.o[0] >= 0 ? y.o[0] + i * y.stride : -1;
    o1 = y.o[1] >= 0 ? y.o[1] + i * y.stride : -1;
}

// psi pairs (psi1, psi2) of a thread's two cells at offsets o0, o1 (-1: no term): one 8-byte
// load or store per psi array when the cells are adjacent and the offset even.
__device__ __forceinline__ void psi_load_pair(const float* p1, const float* p2, int o0, int o1, float2& c0, float2& c1) {
    c0 = c1 = make_float2(0.f, 0.f);
    if (o0 >= 0 && o1 == o0 + 1 && !(o0 & 1)) {
        const float2 u = *reinterpret_cast<const float2*>(p1 + o0);
        const float2 v = *reinterpret_cast<const float2*>(p2 + o0);
        c0 = make_float2(u.x, v.x);
        c1 = make_float2(u.y, v.y);
        return;
    }
    if (o0 >= 0) c0 = make_float2(p1[o0], p2[o0]);
    if (o1 >= 0) c1 = make_float2(p1[o1], p2[o1]);
}

__device__ __forceinline__ void psi_store_pair(float* p1, float* p2, int o0, int o1, float2 c0, float2 c1) {
    if (o0 >= 0 && o1 == o0 + 1 && !(o0 & 1)) {
        *reinterpret_cast<float2*>(p1 + o0) = make_float2(c0.x, c1.x);
        *reinterpret_cast<float2*>(p2 + o0) = make_float2(c0.y, c1.y);
        return;
    }
    if (o0 >= 0) { p1[o0] = c0.x; p2[o0] = c0.y; }
    if (o1 >= 0) { p1[o1] = c1.x; p2[o1] = c1.y; }
}

// The psi pairs of a thread's two cells at one plane, fetched a plane ahead of their use so
// the loads overlap the previous plane's work (the field tiles arrive through the pipeline).
struct PsiPf {
    float2 x[2], y[2], z[2];
    XPlane xp;
};

template <bool HSIDE, bool ZONLY = false>
__device__ __forceinline__ void pml_fetch(const UpdArgs& a, const ZCol& zc, const YCol& yc, int i, int j, int k0,
                                          bool valid, PsiPf& f) {
    int o0, o1;
    zcol_off(zc, i, o0, o1);
    psi_load_pair(zc.p1, zc.p2, o0, o1, f.z[0], f.z[1]);
    if (ZONLY) {  // z terms only (the x and y slabs are corrected by their own launches)
        f.xp.side = -1;
        return;
    }
    ycol_off(yc, i, o0, o1);
    psi_load_pair(yc.p1, yc.p2, o0, o1, f.y[0], f.y[1]);
    xplane_init<HSIDE>(a, i, f.xp);
    o0 = f.xp.side >= 0 && valid ? xplane_off(a, f.xp, j, k0) : -1;
    psi_load_pair(f.xp.p1, f.xp.p2, o0, o0 >= 0 ? o0 + 1 : -1, f.x[0], f.x[1]);
}

// One slab term on axis AX at a cell (ax_term's arithmetic): the differences of the slab
// axis (AX 0: d_x F_z, d_x F_y; AX 1: d_y F_x, d_y F_z; AX 2: d_z F_y, d_z F_x) advance the
// psi pair (reverse steps keep it frozen) and correct two curl components; returns the pair
// a forward step stores.
template <bool REV, int AX>
__device__ __forceinline__ float2 tma_slab_term(float ca, float cb, float km, int kone, float2 pv, const float d[6],
                                                float cu[3]) {
    const float d1 = AX == 0 ? d[3] : (AX == 1 ? d[5] : d[1]);
    const float d2 = AX == 0 ? d[4] : (AX == 1 ? d[0] : d[2]);
    float q1 = pv.x, q2 = pv.y;
    if (!REV) {
        q1 = cb * q1 + ca * d1;
        q2 = cb * q2 + ca * d2;
    }
    float c1 = q1, c2 = q2;
    if (!kone) {
        c1 = km * d1 + q1;
        c2 = km * d2 + q2;
    }
    if (AX == 0) { cu[1] -= c1; cu[2] += c2; }
    else if (AX == 1) { cu[2] -= c1; cu[0] += c2; }
    else { cu[0] -= c1; cu[1] += c2; }
    return make_float2(q1, q2);
}

// The slab terms of cell e (axis order x, y, z); q holds the psi pairs to store.
template <bool REV, bool ZONLY = false>
__device__ __forceinline__ void pml_terms(const PsiPf& f, const YCol& yc, const ZCol& zc, int e, const float d[6],
                                          float cu[3], float2 q[3]) {
    if (!ZONLY && f.xp.side >= 0) q[0] = tma_slab_term<REV, 0>(f.xp.ca, f.xp.cb, f.xp.km, f.xp.kone, f.x[e], d, cu);
    if (!ZONLY && yc.o[e] >= 0) q[1] = tma_slab_term<REV, 1>(yc.ca, yc.cb, yc.km, yc.kone, f.y[e], d, cu);
    if (zc.o[e] >= 0) q[2] = tma_slab_term<REV, 2>(zc.ca[e], zc.cb[e], zc.km[e], zc.kone, f.z[e], d, cu);
}

// The forward step's psi stores of both cells at plane i.
template <bool ZONLY = false>
__device__ __forceinline__ void pml_store(const UpdArgs& a, const PsiPf& f, const YCol& yc, const ZCol& zc, int i, int j,
                                          int k0, const float2 q[2][3]) {
    int o0, o1;
    if (!ZONLY) {
        if (f.xp.side >= 0) {
            o0 = xplane_off(a, f.xp, j, k0);
            psi_store_pair(f.xp.p1, f.xp.p2, o0, o0 + 1, q[0][0], q[1][0]);
        }
        ycol_off(yc, i, o0, o1);
        psi_store_pair(yc.p1, yc.p2, o0, o1, q[0][1], q[1][1]);
    }
    zcol_off(zc, i, o0, o1);
    psi_store_pair(zc.p1, zc.p2, o0, o1, q[0][2], q[1][2]);
}

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n"
        " .reg .pred p;\n"
        " mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
        " selp.u32 %0, 1, 0, p;\n"
        "}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
    for (uint32_t it = 0; it < kWaitLimit; ++it)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 4-D tiled load (z, y, x, component) into shared memory, completing on `bar`.
__device__ __forceinline__ void tma_load4(float* dst, const CUtensorMap* map, uint64_t* bar, int c0, int c1, int c2,
                                          int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// Waits (bounded) for the loads [from, to) that are still in flight, before an early exit.
__device__ __forceinline__ void drain(uint64_t* bar, int ns, int from, int to) {
    for (int p = from; p < to; ++p) mbar_wait_bounded(&bar[p % ns], (uint32_t)((p / ns) & 1));
}

// ---------------------------------------------------------------------------------
// E half-step (forward / reverse), tile loads per plane i:
//   H (3 comps) z in [kt-4, kt+TZ), y in [jt-1, jt+TY)   (backward differences)
//   E, inv_eps, sigma_E on the tile
// Loads cover planes i0-1 .. i1-1; the first only seeds H(i-1) of each column.
// ---------------------------------------------------------------------------------
template <bool REV, int PML = 0>
__global__ void __launch_bounds__(256) k_tma_E(const __grid_constant__ UpdArgs a, const __grid_constant__ CUtensorMap mF,
                                               const __grid_constant__ CUtensorMap mU,
                                               const __grid_constant__ CUtensorMap mM,
                                               const __grid_constant__ CUtensorMap mS, const TmaCfg tc) {
    extern __shared__ __align__(128) float sm[];
    const Geo& g = a.g;
    const int TZ = tc.TZ, TY = tc.TY, NS = tc.ns;
    const int HZ = TZ + 4, HY = TY + 1;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + NS * tc.stage_floats);
    const int tid = threadIdx.x;
    const int half = TZ / 2;
    const int tz = tid % half, ty = tid / half;
    const int kt = a.lo[2] + blockIdx.x * TZ, jt = a.lo[1] + blockIdx.y * TY;
    const int i0 = a.lo[0] + blockIdx.z * a.chunk, i1 = min(i0 + a.chunk, a.hi[0]);
    const int P = i1 - i0 + 1;
    const int k0 = kt + 2 * tz, j = jt + ty;
    const bool valid = k0 < a.hi[2] && j < a.hi[1];
    const long long N = g.N;
    ZCol zc{};
    YCol yc{};
    if (PML) {
        zcol_init<false>(a, j, k0, valid, zc);
        if (PML == 1) ycol_init<false>(a, j, k0, valid, yc);
    }
    if (tc.expire) {  // injected wait expiry: the error path, with no copy issued
        if (tid == 0) atomicExch(tc.err, FDTD_ETIMEOUT);
        return;
    }

    if (tid == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    auto issue = [&](int p) {
        const int s = p % NS;
        const int i = i0 - 1 + p;
        float* st = sm + s * tc.stage_floats;
        mbar_expect_tx(&bar[s], tc.stage_bytes);
        tma_load4(st, &mF, &bar[s], kt - 4, jt - 1, i, 0);
        tma_load4(st + tc.off_U, &mU, &bar[s], kt, jt, i, 0);
        if (tc.nm) tma_load4(st + tc.off_M, &mM, &bar[s], kt, jt, i, 0);
        if (tc.nsig) tma_load4(st + tc.off_S, &mS, &bar[s], kt, jt, i, 0);
    };
    if (tid == 0)
        for (int p = 0; p < min(NS, P); ++p) issue(p);

    float Hy_m[2] = {0.f, 0.f}, Hz_m[2] = {0.f, 0.f};
    PsiPf pf{}, pn{};  // psi of the plane being updated and of the next one
    for (int p = 0; p < P; ++p) {
        const int s = p % NS;
        const int i = i0 - 1 + p;
        if (PML) {
            pf = pn;
            if (p + 1 < P) pml_fetch<false, PML == 2>(a, zc, yc, i + 1, j, k0, valid, pn);
        }
        const bool ok = mbar_wait_bounded(&bar[s], (uint32_t)((p / NS) & 1));
        const float* F = sm + s * tc.stage_floats;
        if (ok && p == 0) {
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                Hy_m[e] = F[(1 * HY + ty + 1) * HZ + 4 + 2 * tz + e];
                Hz_m[e] = F[(2 * HY + ty + 1) * HZ + 4 + 2 * tz + e];
            }
        } else if (ok && valid) {
            const float* U = F + tc.off_U;
            const float* M = F + tc.off_M;
            const float* S = F + tc.off_S;
            const long long c = cell_index(g, i, j, k0);
            float out[3][2];
            float2 qn[2][3];  // the psi pairs a forward step stores
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int kk = 4 + 2 * tz + e;
                const int cz = 2 * tz + e;
                const float Hx = F[(0 * HY + ty + 1) * HZ + kk];
                const float Hy = F[(1 * HY + ty + 1) * HZ + kk];
                const float Hz = F[(2 * HY + ty + 1) * HZ + kk];
                const float Hz_jm = F[(2 * HY + ty) * HZ + kk];
                const float Hx_jm = F[(0 * HY + ty) * HZ + kk];
                const float Hy_km = F[(1 * HY + ty + 1) * HZ + kk - 1];
                const float Hx_km = F[(0 * HY + ty + 1) * HZ + kk - 1];
                const float d[6] = {Hz - Hz_jm, Hy - Hy_km, Hx - Hx_km, Hz - Hz_m[e], Hy - Hy_m[e], Hx - Hx_jm};
                Hy_m[e] = Hy;
                Hz_m[e] = Hz;
                float cu[3] = {d[0] - d[1], d[2] - d[3], d[4] - d[5]};
                if (PML) pml_terms<REV, PML == 2>(pf, yc, zc, e, d, cu, qn[e]);
#pragma unroll
                for (int comp = 0; comp < 3; ++comp) {
                    const float u0 = U[(comp * TY + ty) * TZ + cz];
                    const float m = tc.nm ? M[((tc.nm == 3 ? comp : 0) * TY + ty) * TZ + cz] : a.mat_scalar;
                    float u;
                    if (tc.nsig) {
                        const float sg = S[((tc.nsig == 3 ? comp : 0) * TY + ty) * TZ + cz];
                        const float q = g.c * sg * g.eta0 * m / 2.f;
                        u = REV ? (u0 * (1.f + q) - g.c * cu[comp] * m) / (1.f - q)
                                : ((1.f - q) * u0 + g.c * cu[comp] * m) / (1.f + q);
                    } else {
                        u = REV ? u0 - g.c * cu[comp] * m : u0 + g.c * cu[comp] * m;
                    }
                    if (g.pec && face_zero(g, g.pec, comp, i, j, k0 + e)) u = 0.f;
                    out[comp][e] = u;
                }
            }
#pragma unroll
            for (int comp = 0; comp < 3; ++comp)
                *reinterpret_cast<float2*>(a.Uout + comp * N + c) = make_float2(out[comp][0], out[comp][1]);
            if (PML && !REV) pml_store<PML == 2>(a, pf, yc, zc, i, j, k0, qn);
        }
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(tc.err, FDTD_ETIMEOUT);
                drain(bar, NS, p, min(p + NS, P));
            }
            return;
        }
        if (tid == 0 && p + NS < P) {
            fence_proxy_async();
            issue(p + NS);
        }
    }
}

// ---------------------------------------------------------------------------------
// H half-step (forward / reverse), tile loads per plane i:
//   E (3 comps) z in [kt-4, kt+TZ+4), y in [jt-1, jt+TY+1)   (forward differences and
//   the -y / +z neighbours of the fused detectors' co-location)
//   H, inv_mu, sigma_H on the tile
// Loads cover planes i0 .. i1; plane i is computed once the loads of i and i+1 landed.
// ---------------------------------------------------------------------------------
template <bool REV, int PML = 0>
__global__ void __launch_bounds__(256) k_tma_H(const __grid_constant__ UpdArgs a, const __grid_constant__ CUtensorMap mF,
                                               const __grid_constant__ CUtensorMap mU,
                                               const __grid_constant__ CUtensorMap mM,
                                               const __grid_constant__ CUtensorMap mS,
                                               const __grid_constant__ CUtensorMap mD, const TmaCfg tc) {
    extern __shared__ __align__(128) float sm[];
    const Geo& g = a.g;
    const int TZ = tc.TZ, TY = tc.TY, NS = tc.ns;
    const int EZ = TZ + 8, EY = TY + 2;
    uint64_t* bar = reinterpret_cast<uint64_t*>(sm + NS * tc.stage_floats);
    const int tid = threadIdx.x;
    const int half = TZ / 2;
    const int tz = tid % half, ty = tid / half;
    const int kt = a.lo[2] + blockIdx.x * TZ, jt = a.lo[1] + blockIdx.y * TY;
    const int i0 = a.lo[0] + blockIdx.z * a.chunk, i1 = min(i0 + a.chunk, a.hi[0]);
    const int P = i1 - i0 + 1;
    const int k0 = kt + 2 * tz, j = jt + ty;
    const bool valid = k0 < a.hi[2] && j < a.hi[1];
    const long long N = g.N;
    ZCol zc{};
    YCol yc{};
    if (PML) {
        zcol_init<true>(a, j, k0, valid, zc);
        if (PML == 1) ycol_init<true>(a, j, k0, valid, yc);
    }

    int slot[kMaxFuse];
    float2 w[kMaxFuse][kMaxFuseFreq];
    bool any = false;
#pragma unroll
    for (int q = 0; q < kMaxFuse; ++q) {
        slot[q] = -1;
        if (REV || q >= a.n_fuse) continue;
        const int t = *a.tp;
        slot[q] = __ldg(a.fuse[q].slot + t + 1);
        any |= slot[q] >= 0;
#pragma unroll
        for (int f = 0; f < kMaxFuseFreq; ++f)
            w[q][f] = (slot[q] >= 0 && f < a.fuse[q].nfreq && a.fuse[q].kind == FDTD_DET_PHASOR)
                          ? __ldg(a.fuse[q].w + (long long)(t + 1) * a.fuse[q].nfreq + f)
                          : make_float2(0.f, 0.f);
    }

    if (tc.expire) {  // injected wait expiry: the error path, with no copy issued
        if (tid == 0) atomicExch(tc.err, FDTD_ETIMEOUT);
        return;
    }
    if (tid == 0) {
        for (int s = 0; s < NS; ++s) mbar_init(&bar[s], 1);
        mbar_fence_init();
    }
    __syncthreads();
    auto issue = [&](int p) {
        const int s = p % NS;
        const int i = i0 + p;
        float* st = sm + s * tc.stage_floats;
        mbar_expect_tx(&bar[s], tc.stage_bytes);
        tma_load4(st, &mF, &bar[s], kt - 4, jt - 1, i, 0);
        tma_load4(st + tc.off_U, &mU, &bar[s], kt, jt, i, 0);
        if (tc.nm) tma_load4(st + tc.off_M, &mM, &bar[s], kt, jt, i, 0);
        if (tc.nsig) tma_load4(st + tc.off_S, &mS, &bar[s], kt, jt, i, 0);
        if (tc.nd) tma_load4(st + tc.off_D, &mD, &bar[s], 2 * (kt - tc.dlo[2]), jt - tc.dlo[1], i - tc.dlo[0], 0);
    };
    if (tid == 0)
        for (int p = 0; p < min(NS, P); ++p) issue(p);

    bool ok = mbar_wait_bounded(&bar[0], 0);
    // Ex(i-1) at k and k+1 of this thread's two cells (fused co-location), seeded at the chunk start
    float Exm[3] = {0.f, 0.f, 0.f};
    if (any && valid) {
#pragma unroll
        for (int e = 0; e < 3; ++e) Exm[e] = ld_halo(g, a.F, 0, i0 - 1, j, k0 + e);
    }
    PsiPf pf{}, pn{};  // psi of the plane being updated and of the next one
    if (PML && P > 1) pml_fetch<true, PML == 2>(a, zc, yc, i0, j, k0, valid, pn);
    for (int p = 0; p + 1 < P; ++p) {
        const int s = p % NS, s1 = (p + 1) % NS;
        const int i = i0 + p;
        if (PML) {
            pf = pn;
            if (p + 2 < P) pml_fetch<true, PML == 2>(a, zc, yc, i + 1, j, k0, valid, pn);
        }
        ok = ok && mbar_wait_bounded(&bar[s1], (uint32_t)(((p + 1) / NS) & 1));
        if (ok && valid) {
            const float* E = sm + s * tc.stage_floats;
            const float* E1 = sm + s1 * tc.stage_floats;
            const float* U = E + tc.off_U;
            const float* M = E + tc.off_M;
            const float* S = E + tc.off_S;
            const long long c = cell_index(g, i, j, k0);
            const int r0 = ty + 1;
            float out[3][2];
            float2 qn[2][3];  // the psi pairs a forward step stores
            float Exc[3];
#pragma unroll
            for (int e = 0; e < 3; ++e) Exc[e] = E[(0 * EY + r0) * EZ + 4 + 2 * tz + e];
#pragma unroll
            for (int e = 0; e < 2; ++e) {
                const int kk = 4 + 2 * tz + e;
                const int cz = 2 * tz + e;
                const float Ex = E[(0 * EY + r0) * EZ + kk];
                const float Ey = E[(1 * EY + r0) * EZ + kk];
                const float Ez = E[(2 * EY + r0) * EZ + kk];
                const float Ez_jp = E[(2 * EY + r0 + 1) * EZ + kk];
                const float Ex_jp = E[(0 * EY + r0 + 1) * EZ + kk];
                const float Ey_kp = E[(1 * EY + r0) * EZ + kk + 1];
                const float Ex_kp = E[(0 * EY + r0) * EZ + kk + 1];
                const float Ez_ip = E1[(2 * EY + r0) * EZ + kk];
                const float Ey_ip = E1[(1 * EY + r0) * EZ + kk];
                const float d[6] = {Ez_jp - Ez, Ey_kp - Ey, Ex_kp - Ex, Ez_ip - Ez, Ey_ip - Ey, Ex_jp - Ex};
                float cu[3] = {d[0] - d[1], d[2] - d[3], d[4] - d[5]};
                if (PML) pml_terms<REV, PML == 2>(pf, yc, zc, e, d, cu, qn[e]);
#pragma unroll
                for (int comp = 0; comp < 3; ++comp) {
                    const float u0 = U[(comp * TY + ty) * TZ + cz];
                    const float m = tc.nm ? M[((tc.nm == 3 ? comp : 0) * TY + ty) * TZ + cz] : a.mat_scalar;
                    float u;
                    if (tc.nsig) {
                        const float sg = S[((tc.nsig == 3 ? comp : 0) * TY + ty) * TZ + cz];
                        const float q = g.c * sg / g.eta0 * m / 2.f;
                        u = REV ? (u0 * (1.f + q) + g.c * cu[comp] * m) / (1.f - q)
                                : ((1.f - q) * u0 - g.c * cu[comp] * m) / (1.f + q);
                    } else {
                        u = REV ? u0 + g.c * cu[comp] * m : u0 - g.c * cu[comp] * m;
                    }
                    if (g.pmc && face_zero(g, g.pmc, comp, i, j, k0 + e)) u = 0.f;
                    out[comp][e] = u;
                }
                if (!REV && any) {
                    const float Ey_jm = E[(1 * EY + r0 - 1) * EZ + kk];
                    const float Eykp_jm = E[(1 * EY + r0 - 1) * EZ + kk + 1];
                    const float* staged = tc.nd ? E + tc.off_D + ty * 2 * TZ + 2 * cz : nullptr;
                    if (staged && a.fuse[0].nfreq == 1 && slot[0] >= 0) {
                        // the staged phasor (one frequency) inline: its tile row is the cell's
                        const DFuse& d = a.fuse[0];
                        const int kc = k0 + e;
                        if (i >= d.lo[0] && i < d.hi[0] && j >= d.lo[1] && j < d.hi[1] && kc >= d.lo[2] && kc < d.hi[2]) {
                            float v[3];
                            if (d.exact) {
                                v[0] = (0.5f * (Ex + Exm[e]) + 0.5f * (Ex_kp + Exm[e + 1])) / 2.f;
                                v[1] = (0.5f * (Ey + Ey_jm) + 0.5f * (Ey_kp + Eykp_jm)) / 2.f;
                            } else {
                                v[0] = Ex;
                                v[1] = Ey;
                            }
                            v[2] = Ez;
                            const long long r =
                                ((long long)(i - d.lo[0]) * d.ry + (j - d.lo[1])) * d.rz + (kc - d.lo[2]);
                            float2* st = reinterpret_cast<float2*>(d.state);
                            const float2 w0 = w[0][0];
                            int o = 0;
#pragma unroll
                            for (int comp = 0; comp < 3; ++comp) {
                                if (!(d.mask >> comp & 1)) continue;
                                float2 z = make_float2(staged[o * TY * 2 * TZ], staged[o * TY * 2 * TZ + 1]);
                                if (d.inverse) { z.x -= v[comp] * w0.x; z.y -= v[comp] * w0.y; }
                                else { z.x += v[comp] * w0.x; z.y += v[comp] * w0.y; }
                                st[(long long)o * d.R + r] = z;
                                ++o;
                            }
                        }
                        if (a.n_fuse > 1)
                            fused_detectors(a, slot, w, i, j, k0 + e, Ex, Ex_kp, Exm[e], Exm[e + 1], Ey, Ey_kp, Ey_jm,
                                            Eykp_jm, Ez, nullptr, 0, nullptr, 1);
                    } else {
                        fused_detectors(a, slot, w, i, j, k0 + e, Ex, Ex_kp, Exm[e], Exm[e + 1], Ey, Ey_kp, Ey_jm,
                                        Eykp_jm, Ez, staged, TY * 2 * TZ);
                    }
                }
            }
#pragma unroll
            for (int e = 0; e < 3; ++e) Exm[e] = Exc[e];
#pragma unroll
            for (int comp = 0; comp < 3; ++comp)
                *reinterpret_cast<float2*>(a.Uout + comp * N + c) = make_float2(out[comp][0], out[comp][1]);
            if (PML && !REV) pml_store<PML == 2>(a, pf, yc, zc, i, j, k0, qn);
        }
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicExch(tc.err, FDTD_ETIMEOUT);
                drain(bar, NS, p + 1, min(p + NS, P));
            }
            return;
        }
        if (tid == 0 && p + NS < P) {
            fence_proxy_async();
            issue(p + NS);
        }
    }
}

}  // namespace fdtd
