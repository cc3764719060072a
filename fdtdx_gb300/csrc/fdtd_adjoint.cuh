// Transposed (vector-Jacobian) forward step of the reversible gradient.
//
// The reference differentiates one forward step with jax.vjp at the reverse-reconstructed
// state (fdtdx/fdtd/fdtd.py:215-251) and keeps the cotangent of inv_permittivities, which
// accumulates over the steps because the step passes the array through (fdtd.py:324-333).
// For fixed materials one forward step is linear in (E, H, psi):
//
//   E-step  E1 = (f E + c ie curl_H(H, psiE')) / d,  psiE' = bE psiE + aE dH,  E3 = PEC(E1 + src)
//   H-step  H1 = (g H - c im curl_E(E3, psiH')) / e,  psiH' = bH psiH + aH dE3,  H3 = PMC(H1 + src)
//   detectors sample (E3, H3) and, with exact interpolation, the average (H + H3) / 2
//
// so its transpose is two gather stencils: the transpose of the H-step (k_adj_H: a
// backward-difference gather of lam_H like an E update) and the transpose of the E-step
// (k_adj_E: a forward-difference gather of lam_E like an H update), preceded by the
// transposed detector samples (k_adj_det, a scatter over the detector region).  Sources
// add constants (the reference stops their gradient, tfsf.py:286-304) and drop out.
// d/d inv_eps is taken in k_adj_E from the E-step with curl_H evaluated at the
// reconstructed H and the frozen psi, as jax.vjp evaluates it there.
//
// Cotangents of complex detector states follow torch's convention: for a real loss L the
// cotangent of z is dL/dRe z + i dL/dIm z, so a real sample x entering z as x * w has
// cotangent Re(conj(w) * lam_z).
#pragma once
#include "fdtd_kernels.cuh"

namespace fdtd {

// A box of cells with its own dense (3, bx, by, bz) storage.
struct DBox {
    int lo[3], n[3];
    long long M;       // cells in the box
    float* buf;        // nullptr: empty box
};

__device__ __forceinline__ bool box_local(const DBox& b, int i, int j, int k, long long& q) {
    const int li = i - b.lo[0], lj = j - b.lo[1], lk = k - b.lo[2];
    if ((unsigned)li >= (unsigned)b.n[0] || (unsigned)lj >= (unsigned)b.n[1] || (unsigned)lk >= (unsigned)b.n[2])
        return false;
    q = ((long long)li * b.n[1] + lj) * b.n[2] + lk;
    return true;
}

struct AdjArgs {
    Geo g;
    const float* E;        // reconstructed E at step t
    const float* H;        // reconstructed H at step t
    const float* ie;       // inv_eps (n_eps comps)
    int n_eps;
    const float* im;       // inv_mu (n_mu comps) or nullptr -> im_scalar
    int n_mu;
    float im_scalar;
    const float* sigE;     // conductivities (pre-scaled) or nullptr
    int n_sigE;
    const float* sigH;
    int n_sigH;
    int n_slab;
    DSlab slab[FDTD_MAX_SLABS];
    const float* psiE1[FDTD_MAX_SLABS];  // frozen psi_E of the reconstructed state
    const float* psiE2[FDTD_MAX_SLABS];
    float* lE;             // in: lam E(t+1) (+ detector part); k_adj_H turns it into lam E3 in place
    float* lH;             // lam H(t+1) (+ detector part)
    float* lE_out;         // lam E(t)
    float* lH_out;         // lam H(t)
    const float* lpE[FDTD_MAX_SLABS][2];  // lam psi_E(t+1), lam psi_H(t+1)
    const float* lpH[FDTD_MAX_SLABS][2];
    float* lpE_out[FDTD_MAX_SLABS][2];    // lam psi_E(t), lam psi_H(t)
    float* lpH_out[FDTD_MAX_SLABS][2];
    float* grad_ie;        // (n_eps, N), accumulated; nullptr: not wanted
    DBox hp;               // detector cotangents of H before the H update (added to lam H(t), then cleared)
};

__device__ __forceinline__ float adj_mat(const float* m, int n, float scalar, long long N, int comp, long long c) {
    if (!m) return scalar;
    return __ldg(m + (n == 3 ? comp : 0) * N + c);
}

// Maps a neighbour index with the halo rule; false when it lies in a zero halo.
__device__ __forceinline__ bool wrap_idx(const Geo& g, int& i, int& j, int& k) {
    if (i < 0) { if (!g.px) return false; i += g.nx; } else if (i >= g.nx) { if (!g.px) return false; i -= g.nx; }
    if (j < 0) { if (!g.py) return false; j += g.ny; } else if (j >= g.ny) { if (!g.py) return false; j -= g.ny; }
    if (k < 0) { if (!g.pz) return false; k += g.nz; } else if (k >= g.nz) { if (!g.pz) return false; k -= g.nz; }
    return true;
}

// Cotangents D[6] of the six raw differences of one half-step at cell (i, j, k), in the
// order the forward kernels use: (dy Fz, dz Fy, dz Fx, dx Fz, dx Fy, dy Fx).  HSIDE selects
// the H-step (F = E3, lam = lam H3, PMC, inv_mu, psi_H) or the E-step (F = H, lam = lam E3,
// PEC, inv_eps, psi_E).  lc[comp] is the cotangent of curl[comp]: -c im/e lam (H) or
// c ie/d lam (E).  A CPML slab adds psi' = b psi + a d and curl corrections
// (-c1 on curl[(a+1)%3], +c2 on curl[(a+2)%3], c = psi' (+ (1/kappa - 1) d)), whose
// transposes feed D and, at the centre cell (OUT), the psi cotangent of step t.
template <bool HSIDE, bool OUT>
__device__ __forceinline__ void lam_diff(const AdjArgs& a, int i, int j, int k, float D[6]) {
    const Geo& g = a.g;
#pragma unroll
    for (int q = 0; q < 6; ++q) D[q] = 0.f;
    if (!wrap_idx(g, i, j, k)) return;
    const long long N = g.N;
    const long long c = cell_index(g, i, j, k);
    const float* L = HSIDE ? a.lH : a.lE;
    const int mask = HSIDE ? g.pmc : g.pec;
    float lc[3];
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
        float l1 = L[comp * N + c];
        if (mask && face_zero(g, mask, comp, i, j, k)) l1 = 0.f;
        float m, den = 1.f;
        if (HSIDE) {
            m = adj_mat(a.im, a.n_mu, a.im_scalar, N, comp, c);
            if (a.sigH) den = 1.f + g.c * adj_mat(a.sigH, a.n_sigH, 0.f, N, comp, c) / g.eta0 * m / 2.f;
            lc[comp] = -(g.c * m / den) * l1;
        } else {
            m = adj_mat(a.ie, a.n_eps, 1.f, N, comp, c);
            if (a.sigE) den = 1.f + g.c * adj_mat(a.sigE, a.n_sigE, 0.f, N, comp, c) * g.eta0 * m / 2.f;
            lc[comp] = (g.c * m / den) * l1;
        }
    }
    D[0] = lc[0]; D[1] = -lc[0]; D[2] = lc[1]; D[3] = -lc[1]; D[4] = lc[2]; D[5] = -lc[2];
    const int idx3[3] = {i, j, k};
#pragma unroll
    for (int s = 0; s < FDTD_MAX_SLABS; ++s) {
        if (s >= a.n_slab) break;
        const DSlab& sl = a.slab[s];
        const int l = idx3[sl.axis] - sl.lo;
        if ((unsigned)l >= (unsigned)sl.L) continue;
        const float* co = sl.coef + (HSIDE ? 3 * sl.L : 0);
        const long long p = psi_offset(sl, i, j, k);
        const int ci = (sl.axis + 1) % 3, cj = (sl.axis + 2) % 3;
        const float* const* lp = HSIDE ? a.lpH[s] : a.lpE[s];
        const float t1 = lp[0][p] - lc[ci];  // cotangent of psi1' (state output + correction c1)
        const float t2 = lp[1][p] + lc[cj];
        const float ca = __ldg(co + l);
        float d1 = ca * t1, d2 = ca * t2;
        if (!sl.kappa_one) {
            const float ikm1 = __ldg(co + 2 * sl.L + l) - 1.f;
            d1 -= ikm1 * lc[ci];
            d2 += ikm1 * lc[cj];
        }
        if (sl.axis == 0) { D[3] += d1; D[4] += d2; }
        else if (sl.axis == 1) { D[5] += d1; D[0] += d2; }
        else { D[1] += d1; D[2] += d2; }
        if (OUT) {
            const float cb = __ldg(co + sl.L + l);
            float* const* lo = HSIDE ? a.lpH_out[s] : a.lpE_out[s];
            lo[0][p] = cb * t1;
            lo[1][p] = cb * t2;
        }
    }
}

// Transpose of the H-step: lam E3 = lam E(t+1) + (forward differences)^T lam D.  E3(c)
// enters D(c) with a minus sign and D(c - axis) with a plus sign.
__global__ void __launch_bounds__(256) k_adj_H(const __grid_constant__ AdjArgs a) {
    const Geo& g = a.g;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.N) return;
    const int k = (int)(c % g.nz);
    const int j = (int)((c / g.nz) % g.ny);
    const int i = (int)(c / ((long long)g.nz * g.ny));
    float D[6], Dx[6], Dy[6], Dz[6];
    lam_diff<true, true>(a, i, j, k, D);
    lam_diff<true, false>(a, i - 1, j, k, Dx);
    lam_diff<true, false>(a, i, j - 1, k, Dy);
    lam_diff<true, false>(a, i, j, k - 1, Dz);
    const long long N = g.N;
    a.lE[c] += (Dz[2] - D[2]) + (Dy[5] - D[5]);
    a.lE[N + c] += (Dz[1] - D[1]) + (Dx[4] - D[4]);
    a.lE[2 * N + c] += (Dy[0] - D[0]) + (Dx[3] - D[3]);
}

// curl_H of the reconstructed H at (i, j, k) with the CPML psi advanced from the frozen
// psi_E (psi' = bE psi + aE d, not stored), as the forward E-step evaluates it.
__device__ __forceinline__ void curl_H_at(const AdjArgs& a, int i, int j, int k, float cu[3]) {
    const Geo& g = a.g;
    const float* H = a.H;
    const long long c = cell_index(g, i, j, k);
    const float hx = __ldg(H + c), hy = __ldg(H + g.N + c), hz = __ldg(H + 2 * g.N + c);
    float d[6];
    d[0] = hz - ld_halo(g, H, 2, i, j - 1, k);
    d[1] = hy - ld_halo(g, H, 1, i, j, k - 1);
    d[2] = hx - ld_halo(g, H, 0, i, j, k - 1);
    d[3] = hz - ld_halo(g, H, 2, i - 1, j, k);
    d[4] = hy - ld_halo(g, H, 1, i - 1, j, k);
    d[5] = hx - ld_halo(g, H, 0, i, j - 1, k);
    cu[0] = d[0] - d[1];
    cu[1] = d[2] - d[3];
    cu[2] = d[4] - d[5];
    const int idx3[3] = {i, j, k};
#pragma unroll
    for (int s = 0; s < FDTD_MAX_SLABS; ++s) {
        if (s >= a.n_slab) break;
        const DSlab& sl = a.slab[s];
        const int l = idx3[sl.axis] - sl.lo;
        if ((unsigned)l >= (unsigned)sl.L) continue;
        const float d1 = sl.axis == 0 ? d[3] : (sl.axis == 1 ? d[5] : d[1]);
        const float d2 = sl.axis == 0 ? d[4] : (sl.axis == 1 ? d[0] : d[2]);
        const float* co = sl.coef;
        const long long p = psi_offset(sl, i, j, k);
        const float ca = __ldg(co + l), cb = __ldg(co + sl.L + l);
        float c1 = cb * __ldg(a.psiE1[s] + p) + ca * d1;
        float c2 = cb * __ldg(a.psiE2[s] + p) + ca * d2;
        if (!sl.kappa_one) {
            const float ikm1 = __ldg(co + 2 * sl.L + l) - 1.f;
            c1 += ikm1 * d1;
            c2 += ikm1 * d2;
        }
        if (sl.axis == 0) { cu[1] -= c1; cu[2] += c2; }
        else if (sl.axis == 1) { cu[2] -= c1; cu[0] += c2; }
        else { cu[0] -= c1; cu[1] += c2; }
    }
}

// Transpose of the E-step: lam E(t) = (f/d) PEC(lam E3); lam H(t) = (g/e) PMC(lam H3) +
// (backward differences)^T lam D + the detectors' H-before-update part.  H(c) enters D(c)
// with a plus sign and D(c + axis) with a minus sign.  The inv_eps cotangent of the cell
// is lam E1 . dE1/d ie with dE1/d ie = (c curl - (c sigma eta0 / 2)(E + E1)) / d.
__global__ void __launch_bounds__(256) k_adj_E(const __grid_constant__ AdjArgs a) {
    const Geo& g = a.g;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.N) return;
    const int k = (int)(c % g.nz);
    const int j = (int)((c / g.nz) % g.ny);
    const int i = (int)(c / ((long long)g.nz * g.ny));
    const long long N = g.N;
    float D[6], Dx[6], Dy[6], Dz[6];
    lam_diff<false, true>(a, i, j, k, D);
    lam_diff<false, false>(a, i + 1, j, k, Dx);
    lam_diff<false, false>(a, i, j + 1, k, Dy);
    lam_diff<false, false>(a, i, j, k + 1, Dz);
    float lh[3];
    lh[0] = (D[2] - Dz[2]) + (D[5] - Dy[5]);
    lh[1] = (D[1] - Dz[1]) + (D[4] - Dx[4]);
    lh[2] = (D[0] - Dy[0]) + (D[3] - Dx[3]);
    long long q;
    const bool in_hp = a.hp.buf && box_local(a.hp, i, j, k, q);
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
        float l1 = a.lH[comp * N + c];
        if (g.pmc && face_zero(g, g.pmc, comp, i, j, k)) l1 = 0.f;
        if (a.sigH) {
            const float m = adj_mat(a.im, a.n_mu, a.im_scalar, N, comp, c);
            const float qh = g.c * adj_mat(a.sigH, a.n_sigH, 0.f, N, comp, c) / g.eta0 * m / 2.f;
            l1 *= (1.f - qh) / (1.f + qh);
        }
        float v = l1 + lh[comp];
        if (in_hp) {
            float* hp = a.hp.buf + comp * a.hp.M + q;
            v += *hp;
            *hp = 0.f;
        }
        a.lH_out[comp * N + c] = v;
    }
    float cu[3] = {0.f, 0.f, 0.f};
    if (a.grad_ie) curl_H_at(a, i, j, k, cu);
    float gsum = 0.f;
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
        float l1 = a.lE[comp * N + c];
        if (g.pec && face_zero(g, g.pec, comp, i, j, k)) l1 = 0.f;
        const float m = adj_mat(a.ie, a.n_eps, 1.f, N, comp, c);
        float le = l1, dm = g.c * cu[comp];
        if (a.sigE) {
            const float hs = g.c * adj_mat(a.sigE, a.n_sigE, 0.f, N, comp, c) * g.eta0 / 2.f;
            const float qe = hs * m;
            const float den = 1.f + qe;
            le = l1 * (1.f - qe) / den;
            if (a.grad_ie) {
                const float e0 = __ldg(a.E + comp * N + c);
                const float e1 = ((1.f - qe) * e0 + g.c * cu[comp] * m) / den;
                dm = (g.c * cu[comp] - hs * (e0 + e1)) / den;
            }
        }
        a.lE_out[comp * N + c] = le;
        if (a.grad_ie) {
            if (a.n_eps == 3) a.grad_ie[comp * N + c] += l1 * dm;
            else gsum += l1 * dm;
        }
    }
    if (a.grad_ie && a.n_eps != 3) a.grad_ie[c] += gsum;
}

// ---------------------------------------------------------------------------------
// Detector cotangents.  A detector sample at step t reads the co-located (E3, H3) and,
// with exact interpolation, H before the update (curl.py:86-224 with the (H_prev + H) / 2
// average of update.py:1088-1098).  Its transpose scatters the sample's cotangent back
// through the same stencil: into lam E3 and lam H3 (atomically: neighbouring samples share
// cells) and into the H-before-update box `hp`.  The flux and energy samples are bilinear,
// so their cotangents need the primal (E3, H3): those are read from a snapshot of the
// region (with a one-cell rim, halo rule applied) taken before the reverse step.
// ---------------------------------------------------------------------------------
struct AdjDet {
    DDet d;
    void* lam;      // cotangent of the detector state (its layout)
    DBox snap;      // bilinear detectors: (6, box) primal E3 | H3 over [lo - 1, hi + 1)
};

__device__ __forceinline__ void add_T(const Geo& g, float* F, int comp, int i, int j, int k, float v) {
    if (!wrap_idx(g, i, j, k)) return;
    atomicAdd(F + comp * g.N + cell_index(g, i, j, k), v);
}

__device__ __forceinline__ void add_hp(const Geo& g, const DBox& hp, int comp, int i, int j, int k, float v) {
    if (!hp.buf || !wrap_idx(g, i, j, k)) return;
    long long q;
    if (!box_local(hp, i, j, k, q)) return;  // the box covers every exact detector's stencil
    atomicAdd(hp.buf + comp * hp.M + q, v);
}

// Transpose of `colocate` for the cotangent gv[6] of the sample at (i, j, k).
__device__ void colocate_T(const AdjArgs& a, int exact, int i, int j, int k, const float gv[6]) {
    const Geo& g = a.g;
    if (!exact) {
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            if (gv[q] != 0.f) add_T(g, a.lE, q, i, j, k, gv[q]);
            if (gv[3 + q] != 0.f) add_T(g, a.lH, q, i, j, k, gv[3 + q]);
        }
        return;
    }
    if (gv[0] != 0.f) {
        const float v = 0.25f * gv[0];
        add_T(g, a.lE, 0, i, j, k, v); add_T(g, a.lE, 0, i - 1, j, k, v);
        add_T(g, a.lE, 0, i, j, k + 1, v); add_T(g, a.lE, 0, i - 1, j, k + 1, v);
    }
    if (gv[1] != 0.f) {
        const float v = 0.25f * gv[1];
        add_T(g, a.lE, 1, i, j, k, v); add_T(g, a.lE, 1, i, j - 1, k, v);
        add_T(g, a.lE, 1, i, j, k + 1, v); add_T(g, a.lE, 1, i, j - 1, k + 1, v);
    }
    if (gv[2] != 0.f) add_T(g, a.lE, 2, i, j, k, gv[2]);
    if (gv[3] != 0.f) {
        const float v = 0.25f * gv[3];
        add_T(g, a.lH, 0, i, j, k, v); add_T(g, a.lH, 0, i, j - 1, k, v);
        add_hp(g, a.hp, 0, i, j, k, v); add_hp(g, a.hp, 0, i, j - 1, k, v);
    }
    if (gv[4] != 0.f) {
        const float v = 0.25f * gv[4];
        add_T(g, a.lH, 1, i, j, k, v); add_T(g, a.lH, 1, i - 1, j, k, v);
        add_hp(g, a.hp, 1, i, j, k, v); add_hp(g, a.hp, 1, i - 1, j, k, v);
    }
    if (gv[5] != 0.f) {
        const float v = 0.0625f * gv[5];
#pragma unroll
        for (int dk = 0; dk < 2; ++dk)
#pragma unroll
            for (int dj = 0; dj < 2; ++dj)
#pragma unroll
                for (int di = 0; di < 2; ++di) {
                    add_T(g, a.lH, 2, i - di, j - dj, k + dk, v);
                    add_hp(g, a.hp, 2, i - di, j - dj, k + dk, v);
                }
    }
}

// Primal co-located sample of a bilinear detector from its snapshot (E3, H3) and the
// reconstructed H before the update.
__device__ void colocate_snap(const AdjArgs& a, const AdjDet& x, int i, int j, int k, float v[6]) {
    const Geo& g = a.g;
    const DBox& s = x.snap;
    auto S = [&](int comp, int ii, int jj, int kk) {
        const long long q = ((long long)(ii - s.lo[0]) * s.n[1] + (jj - s.lo[1])) * s.n[2] + (kk - s.lo[2]);
        return s.buf[comp * s.M + q];
    };
    if (!x.d.exact) {
#pragma unroll
        for (int q = 0; q < 6; ++q) v[q] = S(q, i, j, k);
        return;
    }
    auto hav = [&](int comp, int ii, int jj, int kk) { return (ld_halo(g, a.H, comp, ii, jj, kk) + S(3 + comp, ii, jj, kk)) / 2.f; };
    v[0] = (0.5f * (S(0, i, j, k) + S(0, i - 1, j, k)) + 0.5f * (S(0, i, j, k + 1) + S(0, i - 1, j, k + 1))) / 2.f;
    v[1] = (0.5f * (S(1, i, j, k) + S(1, i, j - 1, k)) + 0.5f * (S(1, i, j, k + 1) + S(1, i, j - 1, k + 1))) / 2.f;
    v[2] = S(2, i, j, k);
    v[3] = 0.5f * (hav(0, i, j, k) + hav(0, i, j - 1, k));
    v[4] = 0.5f * (hav(1, i, j, k) + hav(1, i - 1, j, k));
    const float lx = 0.5f * (hav(2, i, j, k) + hav(2, i - 1, j, k));
    const float lxy = 0.5f * (lx + 0.5f * (hav(2, i, j - 1, k) + hav(2, i - 1, j - 1, k)));
    const float ux = 0.5f * (hav(2, i, j, k + 1) + hav(2, i - 1, j, k + 1));
    const float uxy = 0.5f * (ux + 0.5f * (hav(2, i, j - 1, k + 1) + hav(2, i - 1, j - 1, k + 1)));
    v[5] = (lxy + uxy) / 2.f;
}

// Snapshot of (E, H) over a bilinear detector's box, taken from the state at t + 1.
__global__ void k_adj_snap(const Geo g, const DBox s, const int* __restrict__ slot, const int* __restrict__ tp,
                           const float* __restrict__ E, const float* __restrict__ H) {
    const long long q = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= s.M) return;
    if (__ldg(slot + *tp + 1) < 0) return;
    const int lk = (int)(q % s.n[2]);
    const int lj = (int)((q / s.n[2]) % s.n[1]);
    const int li = (int)(q / ((long long)s.n[2] * s.n[1]));
    const int i = s.lo[0] + li, j = s.lo[1] + lj, k = s.lo[2] + lk;
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
        s.buf[comp * s.M + q] = ld_halo(g, E, comp, i, j, k);
        s.buf[(3 + comp) * s.M + q] = ld_halo(g, H, comp, i, j, k);
    }
}

__global__ void __launch_bounds__(kDetBlock) k_adj_det(const __grid_constant__ AdjArgs a, const __grid_constant__ AdjDet x,
                                                       const int* __restrict__ tp) {
    const DDet& d = x.d;
    const Geo& g = a.g;
    const int t = *tp;
    const int slot = __ldg(d.slot + t + 1);
    if (slot < 0) return;
    const long long r = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= d.R) return;
    const int k = d.lo[2] + (int)(r % d.rz);
    const int j = d.lo[1] + (int)((r / d.rz) % d.ry);
    const int i = d.lo[0] + (int)(r / ((long long)d.rz * d.ry));
    float gv[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (d.kind == FDTD_DET_PHASOR || d.kind == FDTD_DET_FIELD) {
        const int nout = __popc(d.comp_mask & 63);
        int q = 0;
        for (int cq = 0; cq < 6; ++cq) {
            if (!(d.comp_mask >> cq & 1)) continue;
            float l = 0.f;
            if (d.kind == FDTD_DET_PHASOR) {
                const float2* wt = d.w + (long long)(t + 1) * d.nfreq;
                for (int fq = 0; fq < d.nfreq; ++fq) {
                    const float2 w = __ldg(wt + fq);
                    float2 z;
                    if (d.reduce) {
                        const float* lam = reinterpret_cast<const float*>(x.lam) + 2 * (fq * nout + q);
                        z = make_float2(lam[0], lam[1]);
                    } else {
                        z = reinterpret_cast<const float2*>(x.lam)[((long long)fq * nout + q) * d.R + r];
                    }
                    l += w.x * z.x + w.y * z.y;
                }
                if (d.reduce) l /= (float)d.R;
                if (d.inverse) l = -l;
            } else {
                float* lam = reinterpret_cast<float*>(x.lam);
                if (d.reduce) {
                    l = lam[(long long)slot * d.ncomp + q] / (float)d.R;
                } else {
                    float* p = lam + ((long long)slot * d.ncomp + q) * d.R + r;
                    l = *p;
                    *p = 0.f;  // the forward step overwrote this entry
                }
            }
            gv[cq] = l;
            ++q;
        }
    } else {
        float* lam = reinterpret_cast<float*>(x.lam);
        float L[3] = {0.f, 0.f, 0.f};
        for (int q = 0; q < d.ncomp; ++q) {
            if (d.reduce) {
                L[q] = lam[(long long)slot * d.ncomp + q] * d.cell_weight;
            } else {
                float* p = lam + ((long long)slot * d.ncomp + q) * d.R + r;
                L[q] = *p;
                *p = 0.f;
            }
        }
        float v[6];
        colocate_snap(a, x, i, j, k, v);
        if (d.kind == FDTD_DET_FLUX) {
            float gS[3] = {0.f, 0.f, 0.f};
            if (d.keep_all) { gS[0] = d.flux_sign * L[0]; gS[1] = d.flux_sign * L[1]; gS[2] = d.flux_sign * L[2]; }
            else gS[d.flux_axis] = d.flux_sign * L[0];
            // S = (Ey Hz - Ez Hy, Ez Hx - Ex Hz, Ex Hy - Ey Hx)
            gv[0] = -gS[1] * v[5] + gS[2] * v[4];
            gv[1] = gS[0] * v[5] - gS[2] * v[3];
            gv[2] = -gS[0] * v[4] + gS[1] * v[3];
            gv[3] = gS[1] * v[2] - gS[2] * v[1];
            gv[4] = -gS[0] * v[2] + gS[2] * v[0];
            gv[5] = gS[0] * v[1] - gS[1] * v[0];
        } else {  // energy 0.5 sum E^2 / ie + 0.5 sum H^2 / im
            const long long c = cell_index(g, i, j, k);
            float gsum = 0.f;
#pragma unroll
            for (int q = 0; q < 3; ++q) {
                const float ie = adj_mat(a.ie, a.n_eps, 1.f, g.N, q, c);
                const float im = adj_mat(a.im, a.n_mu, a.im_scalar, g.N, q, c);
                gv[q] = L[0] * v[q] / ie;
                gv[3 + q] = L[0] * v[3 + q] / im;
                const float ge = -0.5f * L[0] * v[q] * v[q] / (ie * ie);
                if (a.grad_ie) {
                    if (a.n_eps == 3) atomicAdd(a.grad_ie + q * g.N + c, ge);
                    else gsum += ge;
                }
            }
            if (a.grad_ie && a.n_eps != 3) atomicAdd(a.grad_ie + c, gsum);
        }
    }
    colocate_T(a, d.exact, i, j, k, gv);
}

// Clears the cotangent entry a reducing field / flux / energy detector overwrote at step t
// (after every block of k_adj_det has read it).
__global__ void k_adj_det_clear(const DDet d, void* lam, const int* __restrict__ tp) {
    const int slot = __ldg(d.slot + *tp + 1);
    if (slot < 0) return;
    for (int q = threadIdx.x; q < d.ncomp; q += blockDim.x) reinterpret_cast<float*>(lam)[(long long)slot * d.ncomp + q] = 0.f;
}

}  // namespace fdtd
