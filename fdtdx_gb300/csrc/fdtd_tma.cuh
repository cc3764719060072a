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
    // z-slab shell launches (ZP kernels): which z boxes (bit 0: low, bit 1: high; blockIdx.x
    // picks one), the low box's end and the high box's start
    int zsides, zlo, zhi;
};

// ---------------------------------------------------------------------------------
// CPML z-slab terms inside the TMA half-steps (ZP kernels, launched over the two z-slab
// shell boxes of a split grid, whose cells lie in no x or y slab): a thread's two cells
// have a fixed layer of the slab along the whole x-march, so the slab coefficients are
// read once and the psi offset grows by ny * L per plane.  psi is read with plain loads
// issued before the plane's pipeline wait.  Same arithmetic as ax_term on axis 2
// (fdtdx/core/physics/curl.py:284-308, perfectly_matched_layer.py:138-190).
// ---------------------------------------------------------------------------------
struct ZCol {
    int o[2];              // psi offset of each cell at plane 0 (-1: the cell has no z term)
    int stride;            // psi floats per x plane
    float ca[2], cb[2], km[2];
    int kone;
    float* p1;
    float* p2;
};

template <bool HSIDE>
__device__ __forceinline__ void zcol_init(const UpdArgs& a, int side, int j, int k0, bool valid, ZCol& z) {
    const int L = side ? a.axs[2][1].L : a.axs[2][0].L;
    const int lo = side ? a.axs[2][1].lo : a.axs[2][0].lo;
    const float* co = (side ? a.axs[2][1].coef : a.axs[2][0].coef) + (HSIDE ? 3 * L : 0);
    z.kone = side ? a.axs[2][1].kappa_one : a.axs[2][0].kappa_one;
    z.p1 = side ? a.axp[2][1][0] : a.axp[2][0][0];
    z.p2 = side ? a.axp[2][1][1] : a.axp[2][0][1];
    z.stride = a.g.ny * L;
#pragma unroll
    for (int e = 0; e < 2; ++e) {
        const int l = k0 + e - lo;
        z.o[e] = -1;
        z.ca[e] = z.cb[e] = z.km[e] = 0.f;
        if (valid && L > 0 && (unsigned)l < (unsigned)L) {
            z.o[e] = j * L + l;
            z.ca[e] = __ldg(co + l);
            z.cb[e] = __ldg(co + L + l);
            z.km[e] = z.kone ? 0.f : __ldg(co + 2 * L + l) - 1.f;
        }
    }
}

// psi pair of cell e at plane i (zero without a term), loaded ahead of the plane's wait.
__device__ __forceinline__ float2 zcol_load(const ZCol& z, int e, int i) {
    if (z.o[e] < 0) return make_float2(0.f, 0.f);
    const int o = z.o[e] + i * z.stride;
    return make_float2(z.p1[o], z.p2[o]);
}

// The z term of cell e: d1 = d_z F_y, d2 = d_z F_x; curl_x -= c1, curl_y += c2.
template <bool REV>
__device__ __forceinline__ void zcol_apply(const ZCol& z, int e, int i, float2 pv, float d1, float d2, float cu[3]) {
    if (z.o[e] < 0) return;
    float p1 = pv.x, p2 = pv.y;
    if (!REV) {
        p1 = z.cb[e] * p1 + z.ca[e] * d1;
        p2 = z.cb[e] * p2 + z.ca[e] * d2;
        const int o = z.o[e] + i * z.stride;
        z.p1[o] = p1;
        z.p2[o] = p2;
    }
    float c1 = p1, c2 = p2;
    if (!z.kone) {
        c1 = z.km[e] * d1 + p1;
        c2 = z.km[e] * d2 + p2;
    }
    cu[0] -= c1;
    cu[1] += c2;
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
template <bool REV, bool ZP = false>
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
    // ZP: blockIdx.x picks the z-slab box (low box [0, zlo), high box [zhi, nz))
    const int zside = ZP ? (tc.zsides == 3 ? (int)blockIdx.x : tc.zsides >> 1) : 0;
    const int kt = ZP ? (zside ? tc.zhi : 0) : a.lo[2] + blockIdx.x * TZ, jt = a.lo[1] + blockIdx.y * TY;
    const int kend = ZP ? (zside ? g.nz : tc.zlo) : a.hi[2];
    const int i0 = a.lo[0] + blockIdx.z * a.chunk, i1 = min(i0 + a.chunk, a.hi[0]);
    const int P = i1 - i0 + 1;
    const int k0 = kt + 2 * tz, j = jt + ty;
    const bool valid = k0 < kend && j < a.hi[1];
    const long long N = g.N;
    ZCol zc{};
    if (ZP) zcol_init<false>(a, zside, j, k0, valid, zc);
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
    for (int p = 0; p < P; ++p) {
        const int s = p % NS;
        const int i = i0 - 1 + p;
        float2 zv[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        if (ZP && p > 0) {
            zv[0] = zcol_load(zc, 0, i);
            zv[1] = zcol_load(zc, 1, i);
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
                if (ZP) zcol_apply<REV>(zc, e, i, zv[e], d[1], d[2], cu);
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
template <bool REV, bool ZP = false>
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
    const int zside = ZP ? (tc.zsides == 3 ? (int)blockIdx.x : tc.zsides >> 1) : 0;
    const int kt = ZP ? (zside ? tc.zhi : 0) : a.lo[2] + blockIdx.x * TZ, jt = a.lo[1] + blockIdx.y * TY;
    const int kend = ZP ? (zside ? g.nz : tc.zlo) : a.hi[2];
    const int i0 = a.lo[0] + blockIdx.z * a.chunk, i1 = min(i0 + a.chunk, a.hi[0]);
    const int P = i1 - i0 + 1;
    const int k0 = kt + 2 * tz, j = jt + ty;
    const bool valid = k0 < kend && j < a.hi[1];
    const long long N = g.N;
    ZCol zc{};
    if (ZP) zcol_init<true>(a, zside, j, k0, valid, zc);

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
    for (int p = 0; p + 1 < P; ++p) {
        const int s = p % NS, s1 = (p + 1) % NS;
        const int i = i0 + p;
        float2 zv[2] = {make_float2(0.f, 0.f), make_float2(0.f, 0.f)};
        if (ZP) {
            zv[0] = zcol_load(zc, 0, i);
            zv[1] = zcol_load(zc, 1, i);
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
                if (ZP) zcol_apply<REV>(zc, e, i, zv[e], d[1], d[2], cu);
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
