// Device-side data structures and helpers shared by the FDTD kernels (sm_103a).
//
// Layout in HBM: every field is (3, nx, ny, nz) float32, C order, z fastest; the
// component stride is N = nx*ny*nz.  Material arrays are (n, nx, ny, nz) with
// n in {1, 3, 9}; an isotropic array is read through component 0, a full tensor is stored
// row-major (entry (r, c) is component 3 r + c).  A CPML slab's
// psi arrays have the slab's shape: the full domain with `L` cells along the
// slab axis.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "fdtd_gb300.h"

// Loads of data that another block of the same launch may have written.  The per-phase
// kernels are separate launches, so the read-only path (__ldg) and plain loads see every
// earlier write.  A translation unit that runs several phases in one persistent launch (grid
// barriers between them) defines FDTD_COHERENT_LOADS: the read-only path may then not be
// used for anything the launch writes, and its loads are plain (weak) loads, which see the
// other blocks' writes once the barrier's gpu-scope acquire fence has run.
#ifdef FDTD_COHERENT_LOADS
#define FDTD_LDG(p) (*(p))
#define FDTD_LDC(p) (*(p))
#else
#define FDTD_LDG(p) __ldg(p)
#define FDTD_LDC(p) (*(p))
#endif

namespace fdtd {

struct DSlab {
    int axis, lo, L, kappa_one;
    int sx, sy, sz;             // slab dims
    const float* coef;          // device: a_E, b_E, inv_kappa_E, a_H, b_H, inv_kappa_H (each L)
};

struct Geo {
    int nx, ny, nz;
    long long N;                // cells per component
    int px, py, pz;             // periodic (wrap) flags
    float c;                    // Courant number
    float eta0;                 // free-space impedance mu0*c (host-supplied)
    int pec, pmc;               // face masks, bit (2*axis + side)
    // Bloch boundaries (complex fields, held planar: the real parts (3, N) then the imaginary
    // parts (3, N)): bit a of `bloch` marks a Bloch axis with phase exp(i k L) = bc + i bs.
    // A kernel works on one part; a neighbour wrapped across a Bloch axis is multiplied by the
    // phase ('+' side) or its conjugate ('-' side), which mixes in the other part, `pother`
    // floats away, with sign `psign` (-1 for the real part, +1 for the imaginary part).
    int bloch;
    float bc[3], bs[3];
    long long pother;
    float psign;
};

// A detector accumulated inside the H half-step: E components only, so every value
// it needs is final when the H step runs (phasor or time-domain field, no reduction).
struct DFuse {
    int kind;                   // FDTD_DET_PHASOR or FDTD_DET_FIELD
    int exact, mask, nout, nfreq, inverse;
    int lo[3], hi[3];
    int rx, ry, rz;
    long long R;
    const int* slot;
    const float2* w;
    void* state;
};

constexpr int kMaxFuse = 2;
constexpr int kMaxFuseFreq = 4;

// Arguments of one E or H half-step (forward or reverse).
struct UpdArgs {
    Geo g;
    const float* F;             // field differentiated (H for the E step, E for the H step)
    const float* Uin;           // field updated, read
    float* Uout;                // field updated, written (may alias Uin)
    const float* mat;           // inv_eps (E step) or inv_mu (H step); nullptr -> mat_scalar
    int n_mat;
    float mat_scalar;
    const float* sig;           // conductivity (pre-scaled by dx) or nullptr
    int n_sig;
    int n_slab;
    DSlab slab[FDTD_MAX_SLABS];
    float* psi1[FDTD_MAX_SLABS];
    float* psi2[FDTD_MAX_SLABS];
    int chunk;                  // x planes per block (the block marches along x)
    int lo[3], hi[3];           // the box of cells a TMA launch updates
    // the boxes a register-queue launch updates: its 1-D grid is cut into nbox ranges of
    // blocks, box b owning blocks [bstart[b], bstart[b+1]) laid out as (nbx[b] columns) x (x chunks)
    int nbox;
    int blo[6][3], bhi[6][3], bchunk[6], nbx[6], bstart[7];
    int bslab[6];               // per box: bit s set when slab s can reach the box or its one-cell rim
    // per-axis slab table, valid when axt = 1 (every face holds at most one slab and the two
    // slabs of an axis do not overlap): the slab on each axis' low / high face (L = 0: none)
    // and its psi pair, so a cell's CPML terms are found with compile-time axes
    int axt;
    DSlab axs[3][2];
    float* axp[3][2][2];
    const int* tp;              // device time-step counter
    int n_fuse;
    DFuse fuse[kMaxFuse];
};

struct DSource {
    int kind, comp, magnetic, normal, profile;
    int lo[3], hi[3];
    float sign, coef, omega_dt, ramp_inv, t0, inv2s2;
    const float* incE;
    const float* incH;
    const float* offE;
    const float* offH;
    const float* phE;
    const float* phH;
    const float* teff;
    const uint8_t* on;
    const float* etab;          // dispersive scenes: the E side's profile at integer steps (or nullptr)
    int n_etab;
};

struct DDet {
    int kind, comp_mask, exact, reduce, inverse, nfreq, flux_axis, keep_all;
    int ncomp;                  // recorded components (or Poynting components)
    int lo[3], hi[3];
    int rx, ry, rz;
    long long R;                // region cells
    float flux_sign, cell_weight;
    const int* slot;            // device table (n_table)
    const float2* w;            // device table (n_table, nfreq)
    float* partial;             // scratch: (nblocks, ncomp) block partial sums
    int nblocks;
};

__device__ __forceinline__ long long cell_index(const Geo& g, int i, int j, int k) {
    return ((long long)i * g.ny + j) * g.nz + k;
}

// Field value at (i, j, k) with the reference's one-cell halo semantics
// (fdtdx/core/misc.py:615-641): an out-of-range index on a periodic axis wraps,
// otherwise the value is zero.  Only one-cell excursions are ever requested.
// The Bloch phase of one wrap across axis a (from above: exp(i k L); from below: its
// conjugate), composed into (cr, ci) (fdtdx/fdtd/update.py:92-136, bloch.py:59-94).
__device__ __forceinline__ void bloch_turn(const Geo& g, int a, bool from_above, float& cr, float& ci) {
    if (!(g.bloch >> a & 1)) return;
    const float c = g.bc[a], s = from_above ? g.bs[a] : -g.bs[a];
    const float r = cr * c - ci * s;
    ci = cr * s + ci * c;
    cr = r;
}

// A wrapped neighbour's value in this part: Re or Im of (cr + i ci) (v_re + i v_im).
__device__ __forceinline__ float bloch_mix(const Geo& g, const float* __restrict__ f, long long off, float cr, float ci,
                                           float v) {
    if (ci == 0.f && cr == 1.f) return v;
    return cr * v + g.psign * ci * FDTD_LDG(f + g.pother + off);
}

__device__ __forceinline__ float ld_halo(const Geo& g, const float* __restrict__ f, int comp, int i, int j, int k) {
    float cr = 1.f, ci = 0.f;
    if (i < 0) { if (!g.px) return 0.f; i += g.nx; bloch_turn(g, 0, false, cr, ci); }
    else if (i >= g.nx) { if (!g.px) return 0.f; i -= g.nx; bloch_turn(g, 0, true, cr, ci); }
    if (j < 0) { if (!g.py) return 0.f; j += g.ny; bloch_turn(g, 1, false, cr, ci); }
    else if (j >= g.ny) { if (!g.py) return 0.f; j -= g.ny; bloch_turn(g, 1, true, cr, ci); }
    if (k < 0) { if (!g.pz) return 0.f; k += g.nz; bloch_turn(g, 2, false, cr, ci); }
    else if (k >= g.nz) { if (!g.pz) return 0.f; k -= g.nz; bloch_turn(g, 2, true, cr, ci); }
    const long long off = comp * g.N + cell_index(g, i, j, k);
    const float v = FDTD_LDG(f + off);
    return g.bloch ? bloch_mix(g, f, off, cr, ci, v) : v;
}

// ld_halo without branches: the wrapped index is formed with selects and the load always
// issues from a valid address (a one-cell excursion wraps into the grid), so every load of
// a caller can be in flight at once; a zero-halo neighbour reads 0.
__device__ __forceinline__ float ld_halo_sel(const Geo& g, const float* __restrict__ f, int comp, int i, int j, int k) {
    const bool li = i < 0, ui = i >= g.nx, lj = j < 0, uj = j >= g.ny, lk = k < 0, uk = k >= g.nz;
    const bool ok = (!(li || ui) || g.px) && (!(lj || uj) || g.py) && (!(lk || uk) || g.pz);
    const int ii = li ? i + g.nx : (ui ? i - g.nx : i);
    const int jj = lj ? j + g.ny : (uj ? j - g.ny : j);
    const int kk = lk ? k + g.nz : (uk ? k - g.nz : k);
    const long long off = comp * g.N + cell_index(g, ok ? ii : 0, ok ? jj : 0, ok ? kk : 0);
    const float v = FDTD_LDG(f + off);
    if (g.bloch && ok && (li || ui || lj || uj || lk || uk)) {
        float cr = 1.f, ci = 0.f;
        if (li || ui) bloch_turn(g, 0, ui, cr, ci);
        if (lj || uj) bloch_turn(g, 1, uj, cr, ci);
        if (lk || uk) bloch_turn(g, 2, uk, cr, ci);
        return bloch_mix(g, f, off, cr, ci, v);
    }
    return ok ? v : 0.f;
}

// The 3x3 tensor (row-major) of a material array at cell c: n = 9 (the full tensor), 3 (its
// diagonal), 1 (isotropic) or no array (the scalar times the identity).
__device__ __forceinline__ void tensor_at(const float* __restrict__ m, int n, float scalar, long long N, long long c,
                                          float t[9]) {
#pragma unroll
    for (int q = 0; q < 9; ++q) t[q] = 0.f;
    if (!m) {
        t[0] = t[4] = t[8] = scalar;
    } else if (n == 9) {
#pragma unroll
        for (int q = 0; q < 9; ++q) t[q] = FDTD_LDG(m + q * N + c);
    } else if (n == 3) {
        t[0] = FDTD_LDG(m + c);
        t[4] = FDTD_LDG(m + N + c);
        t[8] = FDTD_LDG(m + 2 * N + c);
    } else {
        t[0] = t[4] = t[8] = FDTD_LDG(m + c);
    }
}

// Inverse of a 3x3 matrix by its adjugate (cofactors over the determinant).
__device__ __forceinline__ void inverse3(const float a[9], float r[9]) {
    const float c00 = a[4] * a[8] - a[5] * a[7];
    const float c01 = a[5] * a[6] - a[3] * a[8];
    const float c02 = a[3] * a[7] - a[4] * a[6];
    const float inv_det = 1.f / (a[0] * c00 + a[1] * c01 + a[2] * c02);
    r[0] = c00 * inv_det;
    r[1] = (a[2] * a[7] - a[1] * a[8]) * inv_det;
    r[2] = (a[1] * a[5] - a[2] * a[4]) * inv_det;
    r[3] = c01 * inv_det;
    r[4] = (a[0] * a[8] - a[2] * a[6]) * inv_det;
    r[5] = (a[2] * a[3] - a[0] * a[5]) * inv_det;
    r[6] = c02 * inv_det;
    r[7] = (a[1] * a[6] - a[0] * a[7]) * inv_det;
    r[8] = (a[0] * a[4] - a[1] * a[3]) * inv_det;
}

// Whether component `comp` at (i, j, k) is zeroed by a conductor face in `mask`
// (PEC for E: fdtdx/objects/boundaries/pec.py:71-77; PMC for H: pmc.py:62-76).
__device__ __forceinline__ bool face_zero(const Geo& g, int mask, int comp, int i, int j, int k) {
    if (!mask) return false;
    const int idx[3] = {i, j, k};
    const int n[3] = {g.nx, g.ny, g.nz};
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (a == comp) continue;
        if ((mask & (1 << (2 * a))) && idx[a] == 0) return true;
        if ((mask & (1 << (2 * a + 1))) && idx[a] == n[a] - 1) return true;
    }
    return false;
}

// Temporal profile at tau (in steps) with a reduced carrier phase `phase` (rad):
// SingleFrequencyProfile: clip(tau*dt/(N_startup*T), 0, 1) cos(phase);
// GaussianPulseProfile:   exp(-(tau - t0)^2 dt^2 / (2 sigma^2)) cos(phase).
__device__ __forceinline__ float profile_amp(const DSource& s, float tau, float phase) {
    const float carrier = cosf(phase);
    if (s.profile == FDTD_PROFILE_CW) {
        const float r = fminf(fmaxf(tau * s.ramp_inv, 0.f), 1.f);
        return r * carrier;
    }
    const float d = tau - s.t0;
    return expf(-d * d * s.inv2s2) * carrier;
}

// The tabulated E-side profile of a plane source in a dispersive scene at tau (in steps):
// linear interpolation between integer steps, 0 outside [0, n - 1] (numpy.interp with zero
// fill, fdtdx/objects/sources/tfsf.py:256-261).
__device__ __forceinline__ float table_amp(const DSource& s, float tau) {
    if (!(tau >= 0.f) || tau > (float)(s.n_etab - 1)) return 0.f;
    const int i = (int)tau;
    const float a = FDTD_LDG(s.etab + i);
    const float b = i + 1 < s.n_etab ? FDTD_LDG(s.etab + i + 1) : a;
    return a + (tau - (float)i) * (b - a);
}

template <typename T>
__device__ __forceinline__ T to_storage(float v);
template <>
__device__ __forceinline__ float to_storage<float>(float v) { return v; }
template <>
__device__ __forceinline__ __nv_bfloat16 to_storage<__nv_bfloat16>(float v) { return __float2bfloat16(v); }
template <>
__device__ __forceinline__ __half to_storage<__half>(float v) { return __float2half(v); }

__device__ __forceinline__ float from_storage(float v) { return v; }
__device__ __forceinline__ float from_storage(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float from_storage(__half v) { return __half2float(v); }

}  // namespace fdtd
