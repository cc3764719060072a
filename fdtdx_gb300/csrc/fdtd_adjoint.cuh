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
// reconstructed H and the frozen psi, as jax.vjp evaluates it there; d/d inv_mu in
// k_grad_mu from the H-step with curl_E evaluated at the recomputed E3.
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
    long long other;   // complex (Bloch) fields: floats from this part's box to the other part's
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
    const float* psiH1[FDTD_MAX_SLABS];  // frozen psi_H (read by the inv_mu cotangent only)
    const float* psiH2[FDTD_MAX_SLABS];
    float* lE;             // in: lam E(t+1) (+ detector part); k_adj_H turns it into lam E3 in place
    float* lH;             // lam H(t+1) (+ detector part)
    float* lE_out;         // lam E(t)
    float* lH_out;         // lam H(t)
    const float* lpE[FDTD_MAX_SLABS][2];  // lam psi_E(t+1), lam psi_H(t+1)
    const float* lpH[FDTD_MAX_SLABS][2];
    float* lpE_out[FDTD_MAX_SLABS][2];    // lam psi_E(t), lam psi_H(t)
    float* lpH_out[FDTD_MAX_SLABS][2];
    float* grad_ie;        // (n_eps, N), accumulated; nullptr: not wanted
    float* grad_im;        // (n_mu, N), accumulated; nullptr: not wanted
    DBox hp;               // detector cotangents of H before the H update (added to lam H(t), then cleared)
    // the boxes a launch covers (the layout of UpdArgs' box table, read by column_of)
    int nbox;
    int blo[6][3], bhi[6][3], bchunk[6], nbx[6], bstart[7];
    int bslab[6];          // per box: bit s set when slab s can reach the box or its one-cell rim
    int ax_slab[3][2];     // the slab on each axis' low / high face (-1: none)
    // copies of those slabs (L = 0: none) and their arrays, read with static indices by the
    // fast shell kernels: frozen psi_E, and [H side][axis][face][psi1 / psi2] cotangents
    DSlab axs[3][2];
    const float* axpE[3][2][2];
    const float* axlp[2][3][2][2];
    float* axlpo[2][3][2][2];
    // complex (Bloch) fields: the part this launch transposes (0 real, 1 imaginary), the number
    // of parts, and per slab the floats from this part's psi cotangents to the other part's
    // (the lam fields' offset is g.pother)
    int part, nparts;
    long long lpother[FDTD_MAX_SLABS];
};

// The slab mask of this block's box.
__device__ __forceinline__ int block_slab_mask(const AdjArgs& a) {
    int m = 0;
#pragma unroll
    for (int q = 0; q < 6; ++q)
        if (q < a.nbox && (int)blockIdx.x >= a.bstart[q]) m = a.bslab[q];
    return m;
}

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

// wrap_idx that also returns the Bloch rotation (cr, ci) of the wrap ((1, 0) when no Bloch
// axis is crossed).  The transposed steps gather across a Bloch face with the same rule the
// forward halo loads use (a wrap from below takes the conjugate phase, from above the phase):
// the adjoint of the phase-shifted wrap read is the conjugate-shifted read the other way.
__device__ __forceinline__ bool wrap_turn(const Geo& g, int& i, int& j, int& k, float& cr, float& ci) {
    cr = 1.f;
    ci = 0.f;
    if (i < 0) { if (!g.px) return false; i += g.nx; bloch_turn(g, 0, false, cr, ci); }
    else if (i >= g.nx) { if (!g.px) return false; i -= g.nx; bloch_turn(g, 0, true, cr, ci); }
    if (j < 0) { if (!g.py) return false; j += g.ny; bloch_turn(g, 1, false, cr, ci); }
    else if (j >= g.ny) { if (!g.py) return false; j -= g.ny; bloch_turn(g, 1, true, cr, ci); }
    if (k < 0) { if (!g.pz) return false; k += g.nz; bloch_turn(g, 2, false, cr, ci); }
    else if (k >= g.nz) { if (!g.pz) return false; k -= g.nz; bloch_turn(g, 2, true, cr, ci); }
    return true;
}

// A value of this part's array at `off` seen through a wrap with rotation (cr, ci): the other
// part, `pother` floats away, mixed in with this part's sign.
__device__ __forceinline__ float mix_at(const float* f, long long off, long long pother, float psign, float cr, float ci) {
    const float v = f[off];
    if (ci == 0.f && cr == 1.f) return v;
    return cr * v + psign * ci * f[off + pother];
}

// The slab a cell lies in along one axis: its layer index l (out: -1 when outside).
__device__ __forceinline__ int slab_layer(const DSlab& sl, int i, int j, int k) {
    const int x = sl.axis == 0 ? i : (sl.axis == 1 ? j : k);
    const int l = x - sl.lo;
    return (unsigned)l < (unsigned)sl.L ? l : -1;
}

// Cotangents D[6] of the six raw differences of one half-step at cell (i, j, k) (wrapped
// with the halo rule; zero in a zero halo), in the order the forward kernels use:
// (dy Fz, dz Fy, dz Fx, dx Fz, dx Fy, dy Fx).  HSIDE selects the H-step (F = E3, lam =
// lam H3, PMC, inv_mu, psi_H) or the E-step (F = H, lam = lam E3, PEC, inv_eps, psi_E).
// lc[comp] is the cotangent of curl[comp]: -c im/e lam (H) or c ie/d lam (E).  A CPML slab
// adds psi' = b psi + a d and curl corrections (-c1 on curl[(a+1)%3], +c2 on curl[(a+2)%3],
// c = psi' (+ (1/kappa - 1) d)); their transposes feed D and, when `out` (the cell is the
// caller's own), the psi cotangent of step t.  PML = false: the cell lies in no slab.
template <bool HSIDE, bool PML>
__device__ __forceinline__ void dcell(const AdjArgs& a, int i, int j, int k, bool out, float D[6], int smask = 63) {
    const Geo& g = a.g;
#pragma unroll
    for (int q = 0; q < 6; ++q) D[q] = 0.f;
    float cr, ci;
    if (!wrap_turn(g, i, j, k, cr, ci)) return;
    const long long N = g.N;
    const long long c = cell_index(g, i, j, k);
    const float* L = HSIDE ? a.lH : a.lE;
    const int mask = HSIDE ? g.pmc : g.pec;
    float lc[3];
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
        float l1 = mix_at(L, comp * N + c, g.pother, g.psign, cr, ci);
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
    if (!PML) return;
#pragma unroll
    for (int s = 0; s < FDTD_MAX_SLABS; ++s) {
        if (s >= a.n_slab) break;
        if (!(smask >> s & 1)) continue;
        const DSlab& sl = a.slab[s];
        const int l = slab_layer(sl, i, j, k);
        if (l < 0) continue;
        const float* co = sl.coef + (HSIDE ? 3 * sl.L : 0);
        const long long p = psi_offset(sl, i, j, k);
        const float lci = sl.axis == 0 ? lc[1] : (sl.axis == 1 ? lc[2] : lc[0]);  // curl[(a+1)%3]
        const float lcj = sl.axis == 0 ? lc[2] : (sl.axis == 1 ? lc[0] : lc[1]);  // curl[(a+2)%3]
        const float* lp0 = HSIDE ? a.lpH[s][0] : a.lpE[s][0];
        const float* lp1 = HSIDE ? a.lpH[s][1] : a.lpE[s][1];
        const float t1 = mix_at(lp0, p, a.lpother[s], g.psign, cr, ci) - lci;  // cotangent of psi1' (+ correction c1)
        const float t2 = mix_at(lp1, p, a.lpother[s], g.psign, cr, ci) + lcj;
        const float ca = __ldg(co + l);
        float d1 = ca * t1, d2 = ca * t2;
        if (!sl.kappa_one) {
            const float ikm1 = __ldg(co + 2 * sl.L + l) - 1.f;
            d1 -= ikm1 * lci;
            d2 += ikm1 * lcj;
        }
        if (sl.axis == 0) { D[3] += d1; D[4] += d2; }
        else if (sl.axis == 1) { D[5] += d1; D[0] += d2; }
        else { D[1] += d1; D[2] += d2; }
        if (out) {
            const float cb = __ldg(co + sl.L + l);
            float* o0 = HSIDE ? a.lpH_out[s][0] : a.lpE_out[s][0];
            float* o1 = HSIDE ? a.lpH_out[s][1] : a.lpE_out[s][1];
            o0[p] = cb * t1;
            o1[p] = cb * t2;
        }
    }
}

// Transpose of the H-step: lam E3 = lam E(t+1) + (forward differences)^T D, in place.
// E3(c) enters D(c) with a minus sign and D(c - axis) with a plus sign.  A thread owns VEC
// z cells of one (j) row and marches along +x, carrying D(c - x) in registers.
template <int VEC, bool PML>
__global__ void __launch_bounds__(256) k_adj_H(const __grid_constant__ AdjArgs a) {
    const Geo& g = a.g;
    int j, k0, i0, i1;
    if (!column_of<VEC>(a, j, k0, i0, i1)) return;
    const long long N = g.N;
    const int sm = PML ? block_slab_mask(a) : 0;
    float Dxm[VEC][2];  // D3, D4 at (i - 1)
#pragma unroll
    for (int e = 0; e < VEC; ++e) {
        float D[6];
        dcell<true, PML>(a, i0 - 1, j, k0 + e, false, D, sm);
        Dxm[e][0] = D[3];
        Dxm[e][1] = D[4];
    }
    for (int i = i0; i < i1; ++i) {
        const long long c = cell_index(g, i, j, k0);
        float Dz[6];
        dcell<true, PML>(a, i, j, k0 - 1, false, Dz, sm);
        Vec<VEC> lE[3];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) lE[comp] = ldv_rw<VEC>(a.lE + comp * N + c);
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            float D[6], Dy[6];
            dcell<true, PML>(a, i, j, k0 + e, true, D, sm);
            dcell<true, PML>(a, i, j - 1, k0 + e, false, Dy, sm);
            lE[0].v[e] += (Dz[2] - D[2]) + (Dy[5] - D[5]);
            lE[1].v[e] += (Dz[1] - D[1]) + (Dxm[e][1] - D[4]);
            lE[2].v[e] += (Dy[0] - D[0]) + (Dxm[e][0] - D[3]);
            Dxm[e][0] = D[3];
            Dxm[e][1] = D[4];
#pragma unroll
            for (int q = 0; q < 6; ++q) Dz[q] = D[q];
        }
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) stv<VEC>(a.lE + comp * N + c, lE[comp]);
    }
}

// curl_H of the reconstructed H at (i, j, k) given its six raw differences d[], with the
// CPML psi advanced from the frozen psi_E (psi' = bE psi + aE d, not stored), as the
// forward E-step evaluates it.
__device__ __forceinline__ void curl_H_cpml(const AdjArgs& a, int i, int j, int k, const float d[6], float cu[3],
                                            int smask) {
#pragma unroll
    for (int s = 0; s < FDTD_MAX_SLABS; ++s) {
        if (s >= a.n_slab) break;
        if (!(smask >> s & 1)) continue;
        const DSlab& sl = a.slab[s];
        const int l = slab_layer(sl, i, j, k);
        if (l < 0) continue;
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
// (backward differences)^T D + the detectors' H-before-update part.  H(c) enters D(c) with
// a plus sign and D(c + axis) with a minus sign.  The inv_eps cotangent of the cell is
// lam E1 . dE1/d ie with dE1/d ie = (c curl - (c sigma eta0 / 2)(E + E1)) / d, curl_H taken
// at the reconstructed H (whose x-neighbour below is carried in registers).  Marches along
// +x carrying D(c + x), computed one plane ahead.
template <int VEC, bool PML>
__global__ void __launch_bounds__(256) k_adj_E(const __grid_constant__ AdjArgs a) {
    const Geo& g = a.g;
    int j, k0, i0, i1;
    if (!column_of<VEC>(a, j, k0, i0, i1)) return;
    const long long N = g.N;
    const long long sy = g.nz;
    const float* __restrict__ H = a.H;
    const bool want_grad = a.grad_ie != nullptr;
    const int sm = PML ? block_slab_mask(a) : 0;
    float Dc[VEC][6];  // D at (i, j, k0 + e)
#pragma unroll
    for (int e = 0; e < VEC; ++e) dcell<false, PML>(a, i0, j, k0 + e, true, Dc[e], sm);
    Vec<VEC> Hy_m, Hz_m;
    if (want_grad) {
        Hy_m = ldv_halo<VEC>(g, H, 1, i0 - 1, j, k0);
        Hz_m = ldv_halo<VEC>(g, H, 2, i0 - 1, j, k0);
    }
    for (int i = i0; i < i1; ++i) {
        const long long c = cell_index(g, i, j, k0);
        float Dtop[6];
        dcell<false, PML>(a, i, j, k0 + VEC, false, Dtop, sm);
        Vec<VEC> lh[3], le[3];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            lh[comp] = ldv<VEC>(a.lH + comp * N + c);
            le[comp] = ldv<VEC>(a.lE + comp * N + c);
        }
        Vec<VEC> Hx, Hy, Hz, Hz_jm, Hx_jm;
        float Hy_k = 0.f, Hx_k = 0.f;
        if (want_grad) {
            Hx = ldv<VEC>(H + c); Hy = ldv<VEC>(H + N + c); Hz = ldv<VEC>(H + 2 * N + c);
            Hz_jm = nbv<VEC>(g, H, 2 * N + c - sy, j > 0, 2, i, j - 1, k0);
            Hx_jm = nbv<VEC>(g, H, c - sy, j > 0, 0, i, j - 1, k0);
            Hy_k = nb(g, H, N + c - 1, k0 > 0, 1, i, j, k0 - 1);
            Hx_k = nb(g, H, c - 1, k0 > 0, 0, i, j, k0 - 1);
        }
        Vec<VEC> outH[3], outE[3];
        float gsum[VEC];
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const int k = k0 + e;
            float Dx[6], Dy[6];
            dcell<false, PML>(a, i + 1, j, k, i + 1 < i1, Dx, sm);
            dcell<false, PML>(a, i, j + 1, k, false, Dy, sm);
            const float* Dz = e + 1 < VEC ? Dc[(e + 1) % VEC] : Dtop;
            float lht[3];
            lht[0] = (Dc[e][2] - Dz[2]) + (Dc[e][5] - Dy[5]);
            lht[1] = (Dc[e][1] - Dz[1]) + (Dc[e][4] - Dx[4]);
            lht[2] = (Dc[e][0] - Dy[0]) + (Dc[e][3] - Dx[3]);
            long long q;
            const bool in_hp = a.hp.buf && box_local(a.hp, i, j, k, q);
#pragma unroll
            for (int comp = 0; comp < 3; ++comp) {
                float l1 = lh[comp].v[e];
                if (g.pmc && face_zero(g, g.pmc, comp, i, j, k)) l1 = 0.f;
                if (a.sigH) {
                    const float m = adj_mat(a.im, a.n_mu, a.im_scalar, N, comp, c + e);
                    const float qh = g.c * adj_mat(a.sigH, a.n_sigH, 0.f, N, comp, c + e) / g.eta0 * m / 2.f;
                    l1 *= (1.f - qh) / (1.f + qh);
                }
                float v = l1 + lht[comp];
                if (in_hp) {
                    float* hp = a.hp.buf + comp * a.hp.M + q;
                    v += *hp;
                    *hp = 0.f;
                }
                outH[comp].v[e] = v;
            }
            float cu[3] = {0.f, 0.f, 0.f};
            if (want_grad) {
                const float hy_km = e == 0 ? Hy_k : Hy.v[e - 1];
                const float hx_km = e == 0 ? Hx_k : Hx.v[e - 1];
                const float d[6] = {Hz.v[e] - Hz_jm.v[e], Hy.v[e] - hy_km, Hx.v[e] - hx_km,
                                    Hz.v[e] - Hz_m.v[e], Hy.v[e] - Hy_m.v[e], Hx.v[e] - Hx_jm.v[e]};
                cu[0] = d[0] - d[1];
                cu[1] = d[2] - d[3];
                cu[2] = d[4] - d[5];
                if (PML) curl_H_cpml(a, i, j, k, d, cu, sm);
            }
            gsum[e] = 0.f;
#pragma unroll
            for (int comp = 0; comp < 3; ++comp) {
                float l1 = le[comp].v[e];
                if (g.pec && face_zero(g, g.pec, comp, i, j, k)) l1 = 0.f;
                float lo = l1, dm = g.c * cu[comp];
                if (a.sigE) {
                    const float m = adj_mat(a.ie, a.n_eps, 1.f, N, comp, c + e);
                    const float hs = g.c * adj_mat(a.sigE, a.n_sigE, 0.f, N, comp, c + e) * g.eta0 / 2.f;
                    const float qe = hs * m;
                    const float den = 1.f + qe;
                    lo = l1 * (1.f - qe) / den;
                    if (want_grad) {
                        const float e0 = __ldg(a.E + comp * N + c + e);
                        const float e1 = ((1.f - qe) * e0 + g.c * cu[comp] * m) / den;
                        dm = (g.c * cu[comp] - hs * (e0 + e1)) / den;
                    }
                }
                outE[comp].v[e] = lo;
                if (want_grad) {
                    if (a.n_eps == 3) a.grad_ie[comp * N + c + e] += l1 * dm;
                    else gsum[e] += l1 * dm;
                }
            }
#pragma unroll
            for (int q2 = 0; q2 < 6; ++q2) Dc[e][q2] = Dx[q2];
        }
        if (want_grad && a.n_eps != 3) {
            Vec<VEC> gr = ldv_rw<VEC>(a.grad_ie + c);
#pragma unroll
            for (int e = 0; e < VEC; ++e) gr.v[e] += gsum[e];
            stv<VEC>(a.grad_ie + c, gr);
        }
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            stv<VEC>(a.lH_out + comp * N + c, outH[comp]);
            stv<VEC>(a.lE_out + comp * N + c, outE[comp]);
        }
        if (want_grad) {
            Hy_m = Hy;
            Hz_m = Hz;
        }
    }
}

// ---------------------------------------------------------------------------------
// Slab-free core of the transposed half-steps.  Without CPML terms the difference
// cotangents of a cell are D = (lc0, -lc0, lc1, -lc1, lc2, -lc2), so the transposes are
// curls of the scaled cotangent field lc:
//   transposed H-step  lam E3 += curl_H(lcH),  lcH = -c im / e PMC(lam H3)   (backward differences)
//   transposed E-step  lam H  = (g/e) PMC(lam H3) + curl_E(lcE),  lcE = c ie / d PEC(lam E3)   (forward)
// i.e. the forward E and H updates with the material moved inside the difference.
// ---------------------------------------------------------------------------------

// CPML term of the slab on `axis` at cell (i, j, k) (in range), given the base curl
// cotangents lci = lc[(axis+1)%3] and lcj = lc[(axis+2)%3] there: the slab adds d1 to the
// difference cotangent of d_axis F_j and d2 to that of d_axis F_i, which is the same as
// differencing along `axis` the effective cotangents lc_ci - d1 and lc_cj + d2.  With
// `out` the psi cotangent of step t is written (the cell is the caller's own).
template <bool HSIDE>
__device__ __forceinline__ void slab_term(const AdjArgs& a, int axis, int i, int j, int k, float lci, float lcj,
                                          bool out, float& d1, float& d2, float cr = 1.f, float ci = 0.f) {
    d1 = 0.f;
    d2 = 0.f;
    const int x = axis == 0 ? i : (axis == 1 ? j : k);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const int s = a.ax_slab[axis][side];
        if (s < 0) continue;
        const DSlab& sl = a.slab[s];
        const int l = x - sl.lo;
        if ((unsigned)l >= (unsigned)sl.L) continue;
        const float* co = sl.coef + (HSIDE ? 3 * sl.L : 0);
        const long long p = psi_offset(sl, i, j, k);
        const float* lp0 = HSIDE ? a.lpH[s][0] : a.lpE[s][0];
        const float* lp1 = HSIDE ? a.lpH[s][1] : a.lpE[s][1];
        const float t1 = mix_at(lp0, p, a.lpother[s], a.g.psign, cr, ci) - lci;
        const float t2 = mix_at(lp1, p, a.lpother[s], a.g.psign, cr, ci) + lcj;
        const float ca = __ldg(co + l);
        float e1 = ca * t1, e2 = ca * t2;
        if (!sl.kappa_one) {
            const float ikm1 = __ldg(co + 2 * sl.L + l) - 1.f;
            e1 -= ikm1 * lci;
            e2 += ikm1 * lcj;
        }
        d1 += e1;
        d2 += e2;
        if (out) {
            const float cb = __ldg(co + sl.L + l);
            float* o0 = HSIDE ? a.lpH_out[s][0] : a.lpE_out[s][0];
            float* o1 = HSIDE ? a.lpH_out[s][1] : a.lpE_out[s][1];
            o0[p] = cb * t1;
            o1[p] = cb * t2;
        }
    }
}

// slab_term for the slab table copies: the axis is a compile-time constant, the slab and
// its arrays are read with static indices and psi offsets are 32-bit (same arithmetic).
template <bool HSIDE, int AX>
__device__ __forceinline__ void slab_term_ax(const AdjArgs& a, int i, int j, int k, float lci, float lcj, bool out,
                                             float& d1, float& d2) {
    d1 = 0.f;
    d2 = 0.f;
    const int x = AX == 0 ? i : (AX == 1 ? j : k);
#pragma unroll
    for (int side = 0; side < 2; ++side) {
        const DSlab& sl = a.axs[AX][side];
        const int l = x - sl.lo;
        if ((unsigned)l >= (unsigned)sl.L) continue;
        const float* co = sl.coef + (HSIDE ? 3 * sl.L : 0);
        const int p = ax_off<AX>(sl.lo, sl.sy, sl.sz, i, j, k);
        const float t1 = a.axlp[HSIDE][AX][side][0][p] - lci;
        const float t2 = a.axlp[HSIDE][AX][side][1][p] + lcj;
        const float ca = __ldg(co + l);
        float e1 = ca * t1, e2 = ca * t2;
        if (!sl.kappa_one) {
            const float ikm1 = __ldg(co + 2 * sl.L + l) - 1.f;
            e1 -= ikm1 * lci;
            e2 += ikm1 * lcj;
        }
        d1 += e1;
        d2 += e2;
        if (out) {
            const float cb = __ldg(co + sl.L + l);
            a.axlpo[HSIDE][AX][side][0][p] = cb * t1;
            a.axlpo[HSIDE][AX][side][1][p] = cb * t2;
        }
    }
}

// axis_terms through the slab table copies, for a grid without periodic axes (zero halo).
template <bool HSIDE, int VEC, int AX>
__device__ __forceinline__ void axis_terms_ax(const AdjArgs& a, int i, int j, int k0, Vec<VEC>& lci, Vec<VEC>& lcj,
                                              bool out) {
    const Geo& g = a.g;
#pragma unroll
    for (int e = 0; e < VEC; ++e) {
        const int kk = k0 + e;
        if ((unsigned)i >= (unsigned)g.nx || (unsigned)j >= (unsigned)g.ny || (unsigned)kk >= (unsigned)g.nz) continue;
        float d1, d2;
        slab_term_ax<HSIDE, AX>(a, i, j, kk, lci.v[e], lcj.v[e], out, d1, d2);
        lci.v[e] -= d1;
        lcj.v[e] += d2;
    }
}

// curl_H_cpml through the slab table copies.
__device__ __forceinline__ void curl_H_cpml_ax(const AdjArgs& a, int i, int j, int k, const float d[6], float cu[3]) {
    const int idx[3] = {i, j, k};
#pragma unroll
    for (int ax = 0; ax < 3; ++ax) {
#pragma unroll
        for (int side = 0; side < 2; ++side) {
            const DSlab& sl = a.axs[ax][side];
            const int l = idx[ax] - sl.lo;
            if ((unsigned)l >= (unsigned)sl.L) continue;
            const float d1 = ax == 0 ? d[3] : (ax == 1 ? d[5] : d[1]);
            const float d2 = ax == 0 ? d[4] : (ax == 1 ? d[0] : d[2]);
            const int p = ax == 0 ? ax_off<0>(sl.lo, sl.sy, sl.sz, i, j, k)
                                  : (ax == 1 ? ax_off<1>(sl.lo, sl.sy, sl.sz, i, j, k) : ax_off<2>(sl.lo, sl.sy, sl.sz, i, j, k));
            const float* co = sl.coef;
            const float ca = __ldg(co + l), cb = __ldg(co + sl.L + l);
            float c1 = cb * __ldg(a.axpE[ax][side][0] + p) + ca * d1;
            float c2 = cb * __ldg(a.axpE[ax][side][1] + p) + ca * d2;
            if (!sl.kappa_one) {
                const float ikm1 = __ldg(co + 2 * sl.L + l) - 1.f;
                c1 += ikm1 * d1;
                c2 += ikm1 * d2;
            }
            if (ax == 0) { cu[1] -= c1; cu[2] += c2; }
            else if (ax == 1) { cu[2] -= c1; cu[0] += c2; }
            else { cu[0] -= c1; cu[1] += c2; }
        }
    }
}

// Effective cotangents along `axis` of a VEC row at (i, j, k0) (wrapped with the halo rule;
// rows in a zero halo hold zeros): lci -= d1, lcj += d2 per cell.
template <bool HSIDE, int VEC>
__device__ __forceinline__ void axis_terms(const AdjArgs& a, int axis, int i, int j, int k0, Vec<VEC>& lci,
                                          Vec<VEC>& lcj, bool out) {
#pragma unroll
    for (int e = 0; e < VEC; ++e) {
        int ii = i, jj = j, kk = k0 + e;
        float cr, ci;
        if (!wrap_turn(a.g, ii, jj, kk, cr, ci)) continue;
        float d1, d2;
        slab_term<HSIDE>(a, axis, ii, jj, kk, lci.v[e], lcj.v[e], out, d1, d2, cr, ci);
        lci.v[e] -= d1;
        lcj.v[e] += d2;
    }
}

// lc of one component at cell c = (i, j, k) from the raw cotangent l there.
template <bool HSIDE>
__device__ __forceinline__ float lc_of(const AdjArgs& a, int comp, int i, int j, int k, long long c, float l) {
    const Geo& g = a.g;
    const long long N = g.N;
    const int mask = HSIDE ? g.pmc : g.pec;
    if (mask && face_zero(g, mask, comp, i, j, k)) return 0.f;
    if (HSIDE) {
        const float m = a.im ? __ldg(a.im + (a.n_mu == 3 ? comp * N : 0) + c) : a.im_scalar;
        float den = 1.f;
        if (a.sigH) den = 1.f + g.c * __ldg(a.sigH + (a.n_sigH == 3 ? comp * N : 0) + c) / g.eta0 * m / 2.f;
        return -(g.c * m / den) * l;
    }
    const float m = __ldg(a.ie + (a.n_eps == 3 ? comp * N : 0) + c);
    float den = 1.f;
    if (a.sigE) den = 1.f + g.c * __ldg(a.sigE + (a.n_sigE == 3 ? comp * N : 0) + c) * g.eta0 * m / 2.f;
    return (g.c * m / den) * l;
}

// lc of one component at a neighbour (wrapped with the halo rule; zero in a zero halo).
template <bool HSIDE>
__device__ __forceinline__ float lc_nb(const AdjArgs& a, int comp, int i, int j, int k) {
    float cr, ci;
    if (!wrap_turn(a.g, i, j, k, cr, ci)) return 0.f;
    const long long c = cell_index(a.g, i, j, k);
    const float* L = HSIDE ? a.lH : a.lE;
    return lc_of<HSIDE>(a, comp, i, j, k, c, mix_at(L, comp * a.g.N + c, a.g.pother, a.g.psign, cr, ci));
}

template <bool HSIDE, int VEC>
__device__ __forceinline__ Vec<VEC> lc_vec(const AdjArgs& a, int comp, int i, int j, int k0, long long c,
                                           const Vec<VEC>& l) {
    Vec<VEC> r;
#pragma unroll
    for (int e = 0; e < VEC; ++e) r.v[e] = lc_of<HSIDE>(a, comp, i, j, k0 + e, c + e, l.v[e]);
    return r;
}

// lc of a VEC row one cell away along x or y (all VEC cells share the halo test).
template <bool HSIDE, int VEC>
__device__ __forceinline__ Vec<VEC> lc_row(const AdjArgs& a, int comp, int i, int j, int k0) {
    const Geo& g = a.g;
    Vec<VEC> r;
    float cr, ci;
    if (!wrap_turn(g, i, j, k0, cr, ci)) {
#pragma unroll
        for (int e = 0; e < VEC; ++e) r.v[e] = 0.f;
        return r;
    }
    const long long c = cell_index(g, i, j, k0);
    const float* L = HSIDE ? a.lH : a.lE;
    Vec<VEC> l = ldv<VEC>(L + comp * g.N + c);
    if (ci != 0.f || cr != 1.f) {  // a row wrapped across a Bloch face: the other part mixed in
        const Vec<VEC> o = ldv<VEC>(L + g.pother + comp * g.N + c);
#pragma unroll
        for (int e = 0; e < VEC; ++e) l.v[e] = cr * l.v[e] + g.psign * ci * o.v[e];
    }
    return lc_vec<HSIDE, VEC>(a, comp, i, j, k0, c, l);
}

// Transposed H-step: lam E3 += curl_H(lcH), in place.  PML: the differences along each axis
// use the effective cotangents of that axis' slab (slab_term), so a neighbour needs one
// slab lookup; the psi cotangents of step t are written at the thread's own cells.
template <int VEC, bool PML>
__global__ void __launch_bounds__(256) k_adj_H_core(const __grid_constant__ AdjArgs a) {
    const Geo& g = a.g;
    int j, k0, i0, i1;
    if (!column_of<VEC>(a, j, k0, i0, i1)) return;
    const long long N = g.N;
    Vec<VEC> ly_m = lc_row<true, VEC>(a, 1, i0 - 1, j, k0);  // lc1, lc2 along x at (i - 1)
    Vec<VEC> lz_m = lc_row<true, VEC>(a, 2, i0 - 1, j, k0);
    if (PML) axis_terms<true, VEC>(a, 0, i0 - 1, j, k0, ly_m, lz_m, false);
    for (int i = i0; i < i1; ++i) {
        const long long c = cell_index(g, i, j, k0);
        Vec<VEC> l[3];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) l[comp] = lc_vec<true, VEC>(a, comp, i, j, k0, c, ldv<VEC>(a.lH + comp * N + c));
        Vec<VEC> l0_jm = lc_row<true, VEC>(a, 0, i, j - 1, k0);
        Vec<VEC> l2_jm = lc_row<true, VEC>(a, 2, i, j - 1, k0);
        float l0_km = lc_nb<true>(a, 0, i, j, k0 - 1);
        float l1_km = lc_nb<true>(a, 1, i, j, k0 - 1);
        // effective cotangents along x (l1x, l2x), y (l2y, l0y), z (l0z, l1z)
        Vec<VEC> l1x = l[1], l2x = l[2], l2y = l[2], l0y = l[0], l0z = l[0], l1z = l[1];
        if (PML) {
            axis_terms<true, VEC>(a, 0, i, j, k0, l1x, l2x, true);
            axis_terms<true, VEC>(a, 1, i, j, k0, l2y, l0y, true);
            axis_terms<true, VEC>(a, 2, i, j, k0, l0z, l1z, true);
            axis_terms<true, VEC>(a, 1, i, j - 1, k0, l2_jm, l0_jm, false);
            Vec<1> z0, z1;
            z0.v[0] = l0_km;
            z1.v[0] = l1_km;
            axis_terms<true, 1>(a, 2, i, j, k0 - 1, z0, z1, false);
            l0_km = z0.v[0];
            l1_km = z1.v[0];
        }
        Vec<VEC> lE[3];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) lE[comp] = ldv_rw<VEC>(a.lE + comp * N + c);
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const float a0 = e == 0 ? l0_km : l0z.v[e - 1];
            const float a1 = e == 0 ? l1_km : l1z.v[e - 1];
            lE[0].v[e] += (l2y.v[e] - l2_jm.v[e]) - (l1z.v[e] - a1);
            lE[1].v[e] += (l0z.v[e] - a0) - (l2x.v[e] - lz_m.v[e]);
            lE[2].v[e] += (l1x.v[e] - ly_m.v[e]) - (l0y.v[e] - l0_jm.v[e]);
        }
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) stv<VEC>(a.lE + comp * N + c, lE[comp]);
        ly_m = l1x;
        lz_m = l2x;
    }
}

// Transposed E-step: lam H(t) = (g/e) PMC(lam H3) + curl_E(lcE) (+ detector part),
// lam E(t) = (f/d) PEC(lam E3), and the inv_eps cotangent.  PML: effective cotangents per
// axis as in k_adj_H_core, and curl_H of the gradient with the frozen psi advanced once.
template <int VEC, bool PML>
__global__ void __launch_bounds__(256) k_adj_E_core(const __grid_constant__ AdjArgs a) {
    const Geo& g = a.g;
    int j, k0, i0, i1;
    if (!column_of<VEC>(a, j, k0, i0, i1)) return;
    const long long N = g.N;
    const long long sy = g.nz;
    const float* __restrict__ H = a.H;
    const bool want_grad = a.grad_ie != nullptr;
    const int sm = PML ? block_slab_mask(a) : 0;
    Vec<VEC> l[3];  // lcE at (i)
    {
        const long long c = cell_index(g, i0, j, k0);
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) l[comp] = lc_vec<false, VEC>(a, comp, i0, j, k0, c, ldv<VEC>(a.lE + comp * N + c));
    }
    Vec<VEC> Hy_m, Hz_m;
    if (want_grad) {
        Hy_m = ldv_halo<VEC>(g, H, 1, i0 - 1, j, k0);
        Hz_m = ldv_halo<VEC>(g, H, 2, i0 - 1, j, k0);
    }
    for (int i = i0; i < i1; ++i) {
        const long long c = cell_index(g, i, j, k0);
        Vec<VEC> ln[3];  // lcE at (i + 1)
#pragma unroll
        for (int comp = 1; comp < 3; ++comp) ln[comp] = lc_row<false, VEC>(a, comp, i + 1, j, k0);
        Vec<VEC> l0_jp = lc_row<false, VEC>(a, 0, i, j + 1, k0);
        Vec<VEC> l2_jp = lc_row<false, VEC>(a, 2, i, j + 1, k0);
        float l0_kp = lc_nb<false>(a, 0, i, j, k0 + VEC);
        float l1_kp = lc_nb<false>(a, 1, i, j, k0 + VEC);
        // effective cotangents: along x at (i) and (i+1), along y at (j) and (j+1), along z
        Vec<VEC> l1x = l[1], l2x = l[2], l2y = l[2], l0y = l[0], l0z = l[0], l1z = l[1];
        Vec<VEC> n1x = ln[1], n2x = ln[2];
        if (PML) {
            axis_terms<false, VEC>(a, 0, i, j, k0, l1x, l2x, true);
            axis_terms<false, VEC>(a, 1, i, j, k0, l2y, l0y, true);
            axis_terms<false, VEC>(a, 2, i, j, k0, l0z, l1z, true);
            axis_terms<false, VEC>(a, 0, i + 1, j, k0, n1x, n2x, false);
            axis_terms<false, VEC>(a, 1, i, j + 1, k0, l2_jp, l0_jp, false);
            Vec<1> z0, z1;
            z0.v[0] = l0_kp;
            z1.v[0] = l1_kp;
            axis_terms<false, 1>(a, 2, i, j, k0 + VEC, z0, z1, false);
            l0_kp = z0.v[0];
            l1_kp = z1.v[0];
        }
        Vec<VEC> le[3], lh[3];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            le[comp] = ldv<VEC>(a.lE + comp * N + c);
            lh[comp] = ldv<VEC>(a.lH + comp * N + c);
        }
        Vec<VEC> Hx, Hy, Hz, Hz_jm, Hx_jm;
        float Hy_k = 0.f, Hx_k = 0.f;
        if (want_grad) {
            Hx = ldv<VEC>(H + c); Hy = ldv<VEC>(H + N + c); Hz = ldv<VEC>(H + 2 * N + c);
            Hz_jm = nbv<VEC>(g, H, 2 * N + c - sy, j > 0, 2, i, j - 1, k0);
            Hx_jm = nbv<VEC>(g, H, c - sy, j > 0, 0, i, j - 1, k0);
            Hy_k = nb(g, H, N + c - 1, k0 > 0, 1, i, j, k0 - 1);
            Hx_k = nb(g, H, c - 1, k0 > 0, 0, i, j, k0 - 1);
        }
        Vec<VEC> outH[3], outE[3], gr;
        if (want_grad && a.n_eps != 3) gr = ldv_rw<VEC>(a.grad_ie + c);
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const int k = k0 + e;
            const float b0 = e + 1 < VEC ? l0z.v[(e + 1) % VEC] : l0_kp;
            const float b1 = e + 1 < VEC ? l1z.v[(e + 1) % VEC] : l1_kp;
            float lht[3];
            lht[0] = (l2_jp.v[e] - l2y.v[e]) - (b1 - l1z.v[e]);
            lht[1] = (b0 - l0z.v[e]) - (n2x.v[e] - l2x.v[e]);
            lht[2] = (n1x.v[e] - l1x.v[e]) - (l0_jp.v[e] - l0y.v[e]);
            long long q = 0;
            const bool in_hp = a.hp.buf && box_local(a.hp, i, j, k, q);
#pragma unroll
            for (int comp = 0; comp < 3; ++comp) {
                float l1 = lh[comp].v[e];
                if (g.pmc && face_zero(g, g.pmc, comp, i, j, k)) l1 = 0.f;
                if (a.sigH) {
                    const float m = a.im ? __ldg(a.im + (a.n_mu == 3 ? comp * N : 0) + c + e) : a.im_scalar;
                    const float qh = g.c * __ldg(a.sigH + (a.n_sigH == 3 ? comp * N : 0) + c + e) / g.eta0 * m / 2.f;
                    l1 *= (1.f - qh) / (1.f + qh);
                }
                float v = l1 + lht[comp];
                if (in_hp) {
                    float* hp = a.hp.buf + comp * a.hp.M + q;
                    v += *hp;
                    *hp = 0.f;
                }
                outH[comp].v[e] = v;
            }
            float cu[3] = {0.f, 0.f, 0.f};
            if (want_grad) {
                const float hy_km = e == 0 ? Hy_k : Hy.v[e - 1];
                const float hx_km = e == 0 ? Hx_k : Hx.v[e - 1];
                const float d[6] = {Hz.v[e] - Hz_jm.v[e], Hy.v[e] - hy_km, Hx.v[e] - hx_km,
                                    Hz.v[e] - Hz_m.v[e], Hy.v[e] - Hy_m.v[e], Hx.v[e] - Hx_jm.v[e]};
                cu[0] = d[0] - d[1];
                cu[1] = d[2] - d[3];
                cu[2] = d[4] - d[5];
                if (PML) curl_H_cpml(a, i, j, k, d, cu, sm);
            }
            float gs = 0.f;
#pragma unroll
            for (int comp = 0; comp < 3; ++comp) {
                float l1 = le[comp].v[e];
                if (g.pec && face_zero(g, g.pec, comp, i, j, k)) l1 = 0.f;
                float lo = l1, dm = g.c * cu[comp];
                if (a.sigE) {
                    const float m = __ldg(a.ie + (a.n_eps == 3 ? comp * N : 0) + c + e);
                    const float hs = g.c * __ldg(a.sigE + (a.n_sigE == 3 ? comp * N : 0) + c + e) * g.eta0 / 2.f;
                    const float qe = hs * m;
                    const float den = 1.f + qe;
                    lo = l1 * (1.f - qe) / den;
                    if (want_grad) {
                        const float e0 = __ldg(a.E + comp * N + c + e);
                        const float e1 = ((1.f - qe) * e0 + g.c * cu[comp] * m) / den;
                        dm = (g.c * cu[comp] - hs * (e0 + e1)) / den;
                    }
                }
                outE[comp].v[e] = lo;
                if (want_grad) {
                    if (a.n_eps == 3) a.grad_ie[comp * N + c + e] += l1 * dm;
                    else gs += l1 * dm;
                }
            }
            if (want_grad && a.n_eps != 3) gr.v[e] += gs;
        }
        if (want_grad && a.n_eps != 3) stv<VEC>(a.grad_ie + c, gr);
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            stv<VEC>(a.lH_out + comp * N + c, outH[comp]);
            stv<VEC>(a.lE_out + comp * N + c, outE[comp]);
        }
        // lcE at (i + 1) becomes lcE at (i); its x component was not needed above
        ln[0] = lc_row<false, VEC>(a, 0, i + 1, j, k0);
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) l[comp] = ln[comp];
        if (want_grad) {
            Hy_m = Hy;
            Hz_m = Hz;
        }
    }
}

// ---------------------------------------------------------------------------------
// Fast forms of the core kernels for the common case: the core box lies strictly inside
// the grid (no halo), no conductivity, no PEC/PMC faces and (transposed H-step) a scalar
// inv_mu.  Then lcH = -c im lam H3 is a uniform scale and lcE = c ie lam E3 a pointwise
// product, and lam E(t) = lam E3.  Addresses advance by one x plane per iteration.
// ---------------------------------------------------------------------------------
template <int VEC>
__device__ __forceinline__ Vec<VEC> vmul(const Vec<VEC>& x, const Vec<VEC>& y) {
    Vec<VEC> r;
#pragma unroll
    for (int e = 0; e < VEC; ++e) r.v[e] = x.v[e] * y.v[e];
    return r;
}

template <int VEC>
__global__ void __launch_bounds__(256) k_adj_H_core_s(const __grid_constant__ AdjArgs a) {
    const Geo& g = a.g;
    int j, k0, i0, i1;
    if (!column_of<VEC>(a, j, k0, i0, i1)) return;
    const long long N = g.N;
    const long long sy = g.nz, sx = (long long)g.ny * g.nz;
    const float s = -g.c * a.im_scalar;
    const float* __restrict__ lH = a.lH + cell_index(g, i0, j, k0);
    float* lE = a.lE + cell_index(g, i0, j, k0);
    Vec<VEC> y_m = ldv<VEC>(lH + N - sx), z_m = ldv<VEC>(lH + 2 * N - sx);  // lam H3 y, z at (i - 1)
    for (int i = i0; i < i1; ++i, lH += sx, lE += sx) {
        const Vec<VEC> x = ldv<VEC>(lH), y = ldv<VEC>(lH + N), z = ldv<VEC>(lH + 2 * N);
        const Vec<VEC> x_jm = ldv<VEC>(lH - sy), z_jm = ldv<VEC>(lH + 2 * N - sy);
        const float x_km = __ldg(lH - 1), y_km = __ldg(lH + N - 1);
        Vec<VEC> e0 = ldv_rw<VEC>(lE), e1 = ldv_rw<VEC>(lE + N), e2 = ldv_rw<VEC>(lE + 2 * N);
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const float xk = e == 0 ? x_km : x.v[e - 1];
            const float yk = e == 0 ? y_km : y.v[e - 1];
            e0.v[e] += s * ((z.v[e] - z_jm.v[e]) - (y.v[e] - yk));
            e1.v[e] += s * ((x.v[e] - xk) - (z.v[e] - z_m.v[e]));
            e2.v[e] += s * ((y.v[e] - y_m.v[e]) - (x.v[e] - x_jm.v[e]));
        }
        stv<VEC>(lE, e0);
        stv<VEC>(lE + N, e1);
        stv<VEC>(lE + 2 * N, e2);
        y_m = y;
        z_m = z;
    }
}

template <int VEC>
__global__ void __launch_bounds__(256, 3) k_adj_E_core_s(const __grid_constant__ AdjArgs a) {
    const Geo& g = a.g;
    int j, k0, i0, i1;
    if (!column_of<VEC>(a, j, k0, i0, i1)) return;
    const long long N = g.N;
    const long long sy = g.nz, sx = (long long)g.ny * g.nz;
    const long long c0 = cell_index(g, i0, j, k0);
    const bool iso = a.n_eps != 3;
    const long long mN = iso ? 0 : N;  // component stride of inv_eps
    const float cc = g.c;
    const float* __restrict__ lE = a.lE + c0;
    const float* __restrict__ lH = a.lH + c0;
    const float* __restrict__ ie = a.ie + c0;
    const float* __restrict__ H = a.H + c0;
    float* lEo = a.lE_out + c0;
    float* lHo = a.lH_out + c0;
    float* gr = a.grad_ie ? a.grad_ie + c0 : nullptr;
    // lam E3 and ie lam E3 at (i)
    Vec<VEC> le[3], lc[3];
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
        le[comp] = ldv<VEC>(lE + comp * N);
        lc[comp] = vmul<VEC>(le[comp], ldv<VEC>(ie + comp * mN));
    }
    Vec<VEC> Hy_m, Hz_m;
    if (gr) {
        Hy_m = ldv<VEC>(H + N - sx);
        Hz_m = ldv<VEC>(H + 2 * N - sx);
    }
    for (int i = i0; i < i1; ++i, lE += sx, lH += sx, ie += sx, H += sx, lEo += sx, lHo += sx) {
        Vec<VEC> len[3], lcn[3];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            len[comp] = ldv<VEC>(lE + sx + comp * N);
            lcn[comp] = vmul<VEC>(len[comp], ldv<VEC>(ie + sx + comp * mN));
        }
        const Vec<VEC> x_jp = vmul<VEC>(ldv<VEC>(lE + sy), ldv<VEC>(ie + sy));
        const Vec<VEC> z_jp = vmul<VEC>(ldv<VEC>(lE + 2 * N + sy), ldv<VEC>(ie + 2 * mN + sy));
        const float x_kp = __ldg(lE + VEC) * __ldg(ie + VEC);
        const float y_kp = __ldg(lE + N + VEC) * __ldg(ie + mN + VEC);
        const Vec<VEC> h0 = ldv<VEC>(lH), h1 = ldv<VEC>(lH + N), h2 = ldv<VEC>(lH + 2 * N);
        Vec<VEC> Hx, Hy, Hz, Hz_jm, Hx_jm;
        float Hy_k = 0.f, Hx_k = 0.f;
        Vec<VEC> gv[3];
        if (gr) {
            Hx = ldv<VEC>(H); Hy = ldv<VEC>(H + N); Hz = ldv<VEC>(H + 2 * N);
            Hz_jm = ldv<VEC>(H + 2 * N - sy);
            Hx_jm = ldv<VEC>(H - sy);
            Hy_k = __ldg(H + N - 1);
            Hx_k = __ldg(H - 1);
            if (iso) gv[0] = ldv_rw<VEC>(gr);
            else {
#pragma unroll
                for (int comp = 0; comp < 3; ++comp) gv[comp] = ldv_rw<VEC>(gr + comp * N);
            }
        }
        Vec<VEC> o0, o1, o2;
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const float b0 = e + 1 < VEC ? lc[0].v[(e + 1) % VEC] : x_kp;
            const float b1 = e + 1 < VEC ? lc[1].v[(e + 1) % VEC] : y_kp;
            // curl_E(c ie lam): lc holds ie lam, the factor c is applied to the differences
            o0.v[e] = h0.v[e] + cc * ((z_jp.v[e] - lc[2].v[e]) - (b1 - lc[1].v[e]));
            o1.v[e] = h1.v[e] + cc * ((b0 - lc[0].v[e]) - (lcn[2].v[e] - lc[2].v[e]));
            o2.v[e] = h2.v[e] + cc * ((lcn[1].v[e] - lc[1].v[e]) - (x_jp.v[e] - lc[0].v[e]));
            if (gr) {
                const float hy_km = e == 0 ? Hy_k : Hy.v[e - 1];
                const float hx_km = e == 0 ? Hx_k : Hx.v[e - 1];
                const float cu0 = (Hz.v[e] - Hz_jm.v[e]) - (Hy.v[e] - hy_km);
                const float cu1 = (Hx.v[e] - hx_km) - (Hz.v[e] - Hz_m.v[e]);
                const float cu2 = (Hy.v[e] - Hy_m.v[e]) - (Hx.v[e] - Hx_jm.v[e]);
                if (iso) {
                    gv[0].v[e] += cc * (le[0].v[e] * cu0 + le[1].v[e] * cu1 + le[2].v[e] * cu2);
                } else {
                    gv[0].v[e] += cc * le[0].v[e] * cu0;
                    gv[1].v[e] += cc * le[1].v[e] * cu1;
                    gv[2].v[e] += cc * le[2].v[e] * cu2;
                }
            }
        }
        if (a.hp.buf) {  // detector part of lam H(t)
#pragma unroll
            for (int e = 0; e < VEC; ++e) {
                long long q;
                if (!box_local(a.hp, i, j, k0 + e, q)) continue;
                float* hp = a.hp.buf + q;
                o0.v[e] += hp[0]; hp[0] = 0.f;
                o1.v[e] += hp[a.hp.M]; hp[a.hp.M] = 0.f;
                o2.v[e] += hp[2 * a.hp.M]; hp[2 * a.hp.M] = 0.f;
            }
        }
        stv<VEC>(lHo, o0);
        stv<VEC>(lHo + N, o1);
        stv<VEC>(lHo + 2 * N, o2);
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) stv<VEC>(lEo + comp * N, le[comp]);
        if (gr) {
            if (iso) stv<VEC>(gr, gv[0]);
            else {
#pragma unroll
                for (int comp = 0; comp < 3; ++comp) stv<VEC>(gr + comp * N, gv[comp]);
            }
            gr += sx;
            Hy_m = Hy;
            Hz_m = Hz;
        }
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            le[comp] = len[comp];
            lc[comp] = lcn[comp];
        }
    }
}

// ---------------------------------------------------------------------------------
// Fast forms of the CPML-shell kernels (same conditions as the fast core, except that the
// boxes touch the grid faces: neighbours outside the grid read as the zero halo, the
// reference's CPML boundary; no periodic axis).  The slab terms are the per-axis ones of
// k_adj_H_core / k_adj_E_core.
// ---------------------------------------------------------------------------------
template <int VEC>
__device__ __forceinline__ Vec<VEC> vscale(const Vec<VEC>& x, float s) {
    Vec<VEC> r;
#pragma unroll
    for (int e = 0; e < VEC; ++e) r.v[e] = x.v[e] * s;
    return r;
}

template <int VEC>
__device__ __forceinline__ Vec<VEC> vzero() {
    Vec<VEC> r;
#pragma unroll
    for (int e = 0; e < VEC; ++e) r.v[e] = 0.f;
    return r;
}

template <int VEC>
__global__ void __launch_bounds__(256, VEC == 1 ? 4 : 1) k_adj_H_shell_s(const __grid_constant__ AdjArgs a) {
    const Geo& g = a.g;
    int j, k0, i0, i1;
    if (!column_of<VEC>(a, j, k0, i0, i1)) return;
    const long long N = g.N;
    const long long sy = g.nz, sx = (long long)g.ny * g.nz;
    const float s = -g.c * a.im_scalar;
    const bool jm = j > 0, km = k0 > 0;
    const float* __restrict__ lH = a.lH + cell_index(g, i0, j, k0);
    float* lE = a.lE + cell_index(g, i0, j, k0);
    // lc1, lc2 along x at (i - 1)
    Vec<VEC> y_m = vzero<VEC>(), z_m = vzero<VEC>();
    if (i0 > 0) {
        y_m = vscale<VEC>(ldv<VEC>(lH + N - sx), s);
        z_m = vscale<VEC>(ldv<VEC>(lH + 2 * N - sx), s);
        axis_terms_ax<true, VEC, 0>(a, i0 - 1, j, k0, y_m, z_m, false);
    }
    for (int i = i0; i < i1; ++i, lH += sx, lE += sx) {
        const Vec<VEC> x = vscale<VEC>(ldv<VEC>(lH), s), y = vscale<VEC>(ldv<VEC>(lH + N), s);
        const Vec<VEC> z = vscale<VEC>(ldv<VEC>(lH + 2 * N), s);
        Vec<VEC> x_jm = vzero<VEC>(), z_jm = vzero<VEC>();
        if (jm) {
            x_jm = vscale<VEC>(ldv<VEC>(lH - sy), s);
            z_jm = vscale<VEC>(ldv<VEC>(lH + 2 * N - sy), s);
        }
        Vec<1> x_km, y_km;
        x_km.v[0] = km ? s * __ldg(lH - 1) : 0.f;
        y_km.v[0] = km ? s * __ldg(lH + N - 1) : 0.f;
        Vec<VEC> l1x = y, l2x = z, l2y = z, l0y = x, l0z = x, l1z = y;
        axis_terms_ax<true, VEC, 0>(a, i, j, k0, l1x, l2x, true);
        axis_terms_ax<true, VEC, 1>(a, i, j, k0, l2y, l0y, true);
        axis_terms_ax<true, VEC, 2>(a, i, j, k0, l0z, l1z, true);
        if (jm) axis_terms_ax<true, VEC, 1>(a, i, j - 1, k0, z_jm, x_jm, false);
        if (km) axis_terms_ax<true, 1, 2>(a, i, j, k0 - 1, x_km, y_km, false);
        Vec<VEC> e0 = ldv_rw<VEC>(lE), e1 = ldv_rw<VEC>(lE + N), e2 = ldv_rw<VEC>(lE + 2 * N);
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const float a0 = e == 0 ? x_km.v[0] : l0z.v[e - 1];
            const float a1 = e == 0 ? y_km.v[0] : l1z.v[e - 1];
            e0.v[e] += (l2y.v[e] - z_jm.v[e]) - (l1z.v[e] - a1);
            e1.v[e] += (l0z.v[e] - a0) - (l2x.v[e] - z_m.v[e]);
            e2.v[e] += (l1x.v[e] - y_m.v[e]) - (l0y.v[e] - x_jm.v[e]);
        }
        stv<VEC>(lE, e0);
        stv<VEC>(lE + N, e1);
        stv<VEC>(lE + 2 * N, e2);
        y_m = l1x;
        z_m = l2x;
    }
}

template <int VEC>
__global__ void __launch_bounds__(256, VEC == 1 ? 4 : 1) k_adj_E_shell_s(const __grid_constant__ AdjArgs a) {
    const Geo& g = a.g;
    int j, k0, i0, i1;
    if (!column_of<VEC>(a, j, k0, i0, i1)) return;
    const long long N = g.N;
    const long long sy = g.nz, sx = (long long)g.ny * g.nz;
    const long long c0 = cell_index(g, i0, j, k0);
    const long long mN = a.n_eps == 3 ? N : 0;
    const float cc = g.c;
    const bool jm = j > 0, jp = j + 1 < g.ny, km = k0 > 0, kp = k0 + VEC < g.nz;
    const float* __restrict__ lE = a.lE + c0;
    const float* __restrict__ lH = a.lH + c0;
    const float* __restrict__ ie = a.ie + c0;
    const float* __restrict__ H = a.H + c0;
    float* lEo = a.lE_out + c0;
    float* lHo = a.lH_out + c0;
    float* gr = a.grad_ie ? a.grad_ie + c0 : nullptr;
    // lam E3 and lcE = c ie lam E3 at (i)
    Vec<VEC> le[3], lc[3];
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
        le[comp] = ldv<VEC>(lE + comp * N);
        lc[comp] = vscale<VEC>(vmul<VEC>(le[comp], ldv<VEC>(ie + comp * mN)), cc);
    }
    Vec<VEC> Hy_m = vzero<VEC>(), Hz_m = vzero<VEC>();
    if (gr && i0 > 0) {
        Hy_m = ldv<VEC>(H + N - sx);
        Hz_m = ldv<VEC>(H + 2 * N - sx);
    }
    for (int i = i0; i < i1; ++i, lE += sx, lH += sx, ie += sx, H += sx, lEo += sx, lHo += sx) {
        const bool ip = i + 1 < g.nx;
        Vec<VEC> len[3], lcn[3];
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            len[comp] = ip ? ldv<VEC>(lE + sx + comp * N) : vzero<VEC>();
            lcn[comp] = ip ? vscale<VEC>(vmul<VEC>(len[comp], ldv<VEC>(ie + sx + comp * mN)), cc) : vzero<VEC>();
        }
        Vec<VEC> x_jp = vzero<VEC>(), z_jp = vzero<VEC>();
        if (jp) {
            x_jp = vscale<VEC>(vmul<VEC>(ldv<VEC>(lE + sy), ldv<VEC>(ie + sy)), cc);
            z_jp = vscale<VEC>(vmul<VEC>(ldv<VEC>(lE + 2 * N + sy), ldv<VEC>(ie + 2 * mN + sy)), cc);
        }
        Vec<1> x_kp, y_kp;
        x_kp.v[0] = kp ? cc * __ldg(lE + VEC) * __ldg(ie + VEC) : 0.f;
        y_kp.v[0] = kp ? cc * __ldg(lE + N + VEC) * __ldg(ie + mN + VEC) : 0.f;
        // effective cotangents per axis (centre: psi cotangents of step t written)
        Vec<VEC> l1x = lc[1], l2x = lc[2], l2y = lc[2], l0y = lc[0], l0z = lc[0], l1z = lc[1];
        Vec<VEC> n1x = lcn[1], n2x = lcn[2];
        axis_terms_ax<false, VEC, 0>(a, i, j, k0, l1x, l2x, true);
        axis_terms_ax<false, VEC, 1>(a, i, j, k0, l2y, l0y, true);
        axis_terms_ax<false, VEC, 2>(a, i, j, k0, l0z, l1z, true);
        if (ip) axis_terms_ax<false, VEC, 0>(a, i + 1, j, k0, n1x, n2x, false);
        if (jp) axis_terms_ax<false, VEC, 1>(a, i, j + 1, k0, z_jp, x_jp, false);
        if (kp) axis_terms_ax<false, 1, 2>(a, i, j, k0 + VEC, x_kp, y_kp, false);
        const Vec<VEC> h0 = ldv<VEC>(lH), h1 = ldv<VEC>(lH + N), h2 = ldv<VEC>(lH + 2 * N);
        Vec<VEC> Hx, Hy, Hz, Hz_jm = vzero<VEC>(), Hx_jm = vzero<VEC>();
        float Hy_k = 0.f, Hx_k = 0.f;
        Vec<VEC> gv[3];
        if (gr) {
            Hx = ldv<VEC>(H); Hy = ldv<VEC>(H + N); Hz = ldv<VEC>(H + 2 * N);
            if (jm) {
                Hz_jm = ldv<VEC>(H + 2 * N - sy);
                Hx_jm = ldv<VEC>(H - sy);
            }
            if (km) {
                Hy_k = __ldg(H + N - 1);
                Hx_k = __ldg(H - 1);
            }
            if (!mN) gv[0] = ldv_rw<VEC>(gr);
            else {
#pragma unroll
                for (int comp = 0; comp < 3; ++comp) gv[comp] = ldv_rw<VEC>(gr + comp * N);
            }
        }
        Vec<VEC> o0, o1, o2;
#pragma unroll
        for (int e = 0; e < VEC; ++e) {
            const int k = k0 + e;
            const float b0 = e + 1 < VEC ? l0z.v[(e + 1) % VEC] : x_kp.v[0];
            const float b1 = e + 1 < VEC ? l1z.v[(e + 1) % VEC] : y_kp.v[0];
            o0.v[e] = h0.v[e] + ((z_jp.v[e] - l2y.v[e]) - (b1 - l1z.v[e]));
            o1.v[e] = h1.v[e] + ((b0 - l0z.v[e]) - (n2x.v[e] - l2x.v[e]));
            o2.v[e] = h2.v[e] + ((n1x.v[e] - l1x.v[e]) - (x_jp.v[e] - l0y.v[e]));
            if (gr) {
                const float hy_km = e == 0 ? Hy_k : Hy.v[e - 1];
                const float hx_km = e == 0 ? Hx_k : Hx.v[e - 1];
                const float d[6] = {Hz.v[e] - Hz_jm.v[e], Hy.v[e] - hy_km, Hx.v[e] - hx_km,
                                    Hz.v[e] - Hz_m.v[e], Hy.v[e] - Hy_m.v[e], Hx.v[e] - Hx_jm.v[e]};
                float cu[3] = {d[0] - d[1], d[2] - d[3], d[4] - d[5]};
                curl_H_cpml_ax(a, i, j, k, d, cu);
                if (!mN) {
                    gv[0].v[e] += cc * (le[0].v[e] * cu[0] + le[1].v[e] * cu[1] + le[2].v[e] * cu[2]);
                } else {
                    gv[0].v[e] += cc * le[0].v[e] * cu[0];
                    gv[1].v[e] += cc * le[1].v[e] * cu[1];
                    gv[2].v[e] += cc * le[2].v[e] * cu[2];
                }
            }
        }
        if (a.hp.buf) {  // detector part of lam H(t)
#pragma unroll
            for (int e = 0; e < VEC; ++e) {
                long long q;
                if (!box_local(a.hp, i, j, k0 + e, q)) continue;
                float* hp = a.hp.buf + q;
                o0.v[e] += hp[0]; hp[0] = 0.f;
                o1.v[e] += hp[a.hp.M]; hp[a.hp.M] = 0.f;
                o2.v[e] += hp[2 * a.hp.M]; hp[2 * a.hp.M] = 0.f;
            }
        }
        stv<VEC>(lHo, o0);
        stv<VEC>(lHo + N, o1);
        stv<VEC>(lHo + 2 * N, o2);
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) stv<VEC>(lEo + comp * N, le[comp]);
        if (gr) {
            if (!mN) stv<VEC>(gr, gv[0]);
            else {
#pragma unroll
                for (int comp = 0; comp < 3; ++comp) stv<VEC>(gr + comp * N, gv[comp]);
            }
            gr += sx;
            Hy_m = Hy;
            Hz_m = Hz;
        }
#pragma unroll
        for (int comp = 0; comp < 3; ++comp) {
            le[comp] = len[comp];
            lc[comp] = lcn[comp];
        }
    }
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

// The transpose of a wrapped read v_p = cr F_p + psign ci F_q scatters into both parts.
__device__ __forceinline__ void add_T(const Geo& g, float* F, int comp, int i, int j, int k, float v) {
    float cr, ci;
    if (!wrap_turn(g, i, j, k, cr, ci)) return;
    const long long off = comp * g.N + cell_index(g, i, j, k);
    if (ci == 0.f && cr == 1.f) {
        atomicAdd(F + off, v);
        return;
    }
    atomicAdd(F + off, cr * v);
    atomicAdd(F + off + g.pother, g.psign * ci * v);
}

__device__ __forceinline__ void add_hp(const Geo& g, const DBox& hp, int comp, int i, int j, int k, float v) {
    float cr, ci;
    if (!hp.buf || !wrap_turn(g, i, j, k, cr, ci)) return;
    long long q;
    if (!box_local(hp, i, j, k, q)) return;  // the box covers every exact detector's stencil
    if (ci == 0.f && cr == 1.f) {
        atomicAdd(hp.buf + comp * hp.M + q, v);
        return;
    }
    atomicAdd(hp.buf + comp * hp.M + q, cr * v);
    atomicAdd(hp.buf + hp.other + comp * hp.M + q, g.psign * ci * v);
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
    auto hav = [&](int comp, int ii, int jj, int kk) { return (ld_halo_sel(g, a.H, comp, ii, jj, kk) + S(3 + comp, ii, jj, kk)) / 2.f; };
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
    // complex (Bloch) fields: a field detector records the real parts only; a phasor the
    // complex sample (v_re + i v_im) w, whose imaginary part's cotangent is Im(lam) w_re -
    // Re(lam) w_im; per-cell field, flux and energy entries are cleared by the last part
    const bool last = a.part == a.nparts - 1;
    if (d.kind == FDTD_DET_FIELD && a.part != 0) return;
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
                    l += a.part ? w.x * z.y - w.y * z.x : w.x * z.x + w.y * z.y;
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
                if (last) *p = 0.f;
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
            float gsum = 0.f, msum = 0.f;
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
                const float gm = -0.5f * L[0] * v[3 + q] * v[3 + q] / (im * im);
                if (a.grad_im) {
                    if (a.n_mu == 3) atomicAdd(a.grad_im + q * g.N + c, gm);
                    else msum += gm;
                }
            }
            if (a.grad_ie && a.n_eps != 3) atomicAdd(a.grad_ie + c, gsum);
            if (a.grad_im && a.n_mu != 3) atomicAdd(a.grad_im + c, msum);
        }
    }
    colocate_T(a, d.exact, i, j, k, gv);
}

// ---------------------------------------------------------------------------------
// inv_mu cotangent of one forward H-step, H1 = (g H - c im curl_E(E3', psiH')) / e, taken
// as jax.vjp takes it at the reconstructed state (fdtdx/fdtd/fdtd.py:228-249, cotangent
// cot[6] returned at :331): E3' is the E-step recomputed from the reconstructed (E, H)
// and psiH' = bH psiH + aH dE3' is advanced from the frozen psi_H.  The reverse E-step
// inverted the E-step with the frozen psi_E, so E3' equals the state's E3 outside the
// E-slabs and, inside them, E3 + (c ie / d)(psiE' - psiE) on each corrected component
// (psiE' = bE psiE + aE dH, the kappa terms cancel; PEC components stay zero).
// k_grad_mu runs between the reverse H-step (H holds H(t)) and the reverse E-step (E
// still holds E3), after the detector cotangents have been added to lam H3:
//   d im += PMC(lam H3) . dH1/d im,  dH1/d im = (-c curl - (c sigma_H / 2 eta0)(H + H1)) / e.
// ---------------------------------------------------------------------------------

// E3' at (i, j, k) (halo rule: zero in a zero halo).
template <bool PML>
__device__ __forceinline__ float e3_recomputed(const AdjArgs& a, int i, int j, int k, int comp) {
    const Geo& g = a.g;
    if (!wrap_idx(g, i, j, k)) return 0.f;
    const long long N = g.N;
    const long long c = cell_index(g, i, j, k);
    const float v = __ldg(a.E + comp * N + c);
    if (!PML) return v;
    float dc = 0.f;
#pragma unroll
    for (int s = 0; s < FDTD_MAX_SLABS; ++s) {
        if (s >= a.n_slab) break;
        const DSlab& sl = a.slab[s];
        const int ax = sl.axis;
        const int ci = (ax + 1) % 3, cj = (ax + 2) % 3;
        if (comp != ci && comp != cj) continue;
        const int l = slab_layer(sl, i, j, k);
        if (l < 0) continue;
        const int pi = i - (ax == 0), pj = j - (ax == 1), pk = k - (ax == 2);
        const float ca = __ldg(sl.coef + l), cb = __ldg(sl.coef + sl.L + l);
        const long long p = psi_offset(sl, i, j, k);
        if (comp == ci) {  // curl[ci] -= c1, c1 from psi1 and d1 = d_ax H[cj]
            const float d1 = __ldg(a.H + cj * N + c) - ld_halo(g, a.H, cj, pi, pj, pk);
            dc -= (cb - 1.f) * __ldg(a.psiE1[s] + p) + ca * d1;
        } else {           // curl[cj] += c2, c2 from psi2 and d2 = d_ax H[ci]
            const float d2 = __ldg(a.H + ci * N + c) - ld_halo(g, a.H, ci, pi, pj, pk);
            dc += (cb - 1.f) * __ldg(a.psiE2[s] + p) + ca * d2;
        }
    }
    if (dc == 0.f || (g.pec && face_zero(g, g.pec, comp, i, j, k))) return v;
    const float m = adj_mat(a.ie, a.n_eps, 1.f, N, comp, c);
    float den = 1.f;
    if (a.sigE) den = 1.f + g.c * adj_mat(a.sigE, a.n_sigE, 0.f, N, comp, c) * g.eta0 * m / 2.f;
    return v + g.c * m / den * dc;
}

// One thread per cell (z fastest).
template <bool PML>
__global__ void __launch_bounds__(256) k_grad_mu(const __grid_constant__ AdjArgs a) {
    const Geo& g = a.g;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.N) return;
    const long long N = g.N;
    const int k = (int)(c % g.nz);
    const int j = (int)((c / g.nz) % g.ny);
    const int i = (int)(c / ((long long)g.nz * g.ny));
    const float Ex = e3_recomputed<PML>(a, i, j, k, 0);
    const float Ey = e3_recomputed<PML>(a, i, j, k, 1);
    const float Ez = e3_recomputed<PML>(a, i, j, k, 2);
    // raw forward differences in the order (dy Ez, dz Ey, dz Ex, dx Ez, dx Ey, dy Ex)
    const float d[6] = {e3_recomputed<PML>(a, i, j + 1, k, 2) - Ez, e3_recomputed<PML>(a, i, j, k + 1, 1) - Ey,
                        e3_recomputed<PML>(a, i, j, k + 1, 0) - Ex, e3_recomputed<PML>(a, i + 1, j, k, 2) - Ez,
                        e3_recomputed<PML>(a, i + 1, j, k, 1) - Ey, e3_recomputed<PML>(a, i, j + 1, k, 0) - Ex};
    float cu[3] = {d[0] - d[1], d[2] - d[3], d[4] - d[5]};
    if (PML) {
#pragma unroll
        for (int s = 0; s < FDTD_MAX_SLABS; ++s) {
            if (s >= a.n_slab) break;
            const DSlab& sl = a.slab[s];
            const int l = slab_layer(sl, i, j, k);
            if (l < 0) continue;
            const float d1 = sl.axis == 0 ? d[3] : (sl.axis == 1 ? d[5] : d[1]);
            const float d2 = sl.axis == 0 ? d[4] : (sl.axis == 1 ? d[0] : d[2]);
            const float* co = sl.coef + 3 * sl.L;
            const long long p = psi_offset(sl, i, j, k);
            const float ca = __ldg(co + l), cb = __ldg(co + sl.L + l);
            float c1 = cb * __ldg(a.psiH1[s] + p) + ca * d1;
            float c2 = cb * __ldg(a.psiH2[s] + p) + ca * d2;
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
    float gsum = 0.f;
#pragma unroll
    for (int comp = 0; comp < 3; ++comp) {
        float l3 = a.lH[comp * N + c];
        if (g.pmc && face_zero(g, g.pmc, comp, i, j, k)) l3 = 0.f;
        float dm = -g.c * cu[comp];
        if (a.sigH) {
            const float m = adj_mat(a.im, a.n_mu, a.im_scalar, N, comp, c);
            const float hs = g.c * adj_mat(a.sigH, a.n_sigH, 0.f, N, comp, c) / g.eta0 / 2.f;
            const float qh = hs * m;
            const float h0 = __ldg(a.H + comp * N + c);
            const float h1 = ((1.f - qh) * h0 - g.c * m * cu[comp]) / (1.f + qh);
            dm = (-g.c * cu[comp] - hs * (h0 + h1)) / (1.f + qh);
        }
        if (a.n_mu == 3) a.grad_im[comp * N + c] += l3 * dm;
        else gsum += l3 * dm;
    }
    if (a.n_mu != 3) a.grad_im[c] += gsum;
}

// Clears the cotangent entry a reducing field / flux / energy detector overwrote at step t
// (after every block of k_adj_det has read it).
__global__ void k_adj_det_clear(const DDet d, void* lam, const int* __restrict__ tp) {
    const int slot = __ldg(d.slot + *tp + 1);
    if (slot < 0) return;
    for (int q = threadIdx.x; q < d.ncomp; q += blockDim.x) reinterpret_cast<float*>(lam)[(long long)slot * d.ncomp + q] = 0.f;
}

// Transpose of the ADE part of the E-step at t (k_ade folded into the E update,
// fdtdx/fdtd/update.py:316-350), after the transposed E-step has written lam E(t):
// E_new = (f E + c curl inv + inv sum_p (Pc_p - P_hat_p)) / d, P_hat_p = c1 Pc_p + c2 Pp_p + c3 E,
// new Pc = P_hat, new Pp = Pc.  With lam the cotangent of E_new (conductor faces zeroed),
// w = inv / d and lamPc', lamPp' the cotangents of the new pair:
//   lam E(t)   += sum_p c3_p (lamPc'_p - w lam)
//   lam Pc(t)_p = w (1 - c1_p) lam + c1_p lamPc'_p + lamPp'_p
//   lam Pp(t)_p = c2_p (lamPc'_p - w lam)
//   d/d inv    += lam sum_p (Pc_p - P_hat_p) / d^2   (the part the transposed E-step lacks)
// One thread per component and cell; E, Pc, Pp the stored state of step t.
__global__ void __launch_bounds__(256) k_ade_T(const Geo g, const float* __restrict__ lamE3, float* lamE_out,
                                               const float* __restrict__ lPc1, const float* __restrict__ lPp1,
                                               float* __restrict__ lPc0, float* __restrict__ lPp0,
                                               const float* __restrict__ E, const float* __restrict__ Pc,
                                               const float* __restrict__ Pp, const float* __restrict__ c1,
                                               const float* __restrict__ c2, const float* __restrict__ c3, int np,
                                               int nd, const float* __restrict__ ie, int n_eps,
                                               const float* __restrict__ sig, int n_sig, float* grad) {
    const long long N = g.N;
    const long long idx = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= 3 * N) return;
    const int comp = (int)(idx / N);
    const long long c = idx - comp * N;
    const int k = (int)(c % g.nz);
    const long long r = c / g.nz;
    const int j = (int)(r % g.ny);
    const int i = (int)(r / g.ny);
    float lam = lamE3[idx];
    if (g.pec && face_zero(g, g.pec, comp, i, j, k)) lam = 0.f;
    const float m = __ldg(ie + (n_eps == 3 ? comp : 0) * N + c);
    const float d = sig ? 1.f + g.c * __ldg(sig + (n_sig == 3 ? comp : 0) * N + c) * g.eta0 * m / 2.f : 1.f;
    const float w = m / d;
    const float e = __ldg(E + idx);
    float addE = 0.f, dsum = 0.f;
    for (int p = 0; p < np; ++p) {
        const long long pi = ((long long)p * 3 + comp) * N + c;
        const long long ci = ((long long)p * nd + (nd == 3 ? comp : 0)) * N + c;
        const float a1 = __ldg(c1 + ci), a2 = __ldg(c2 + ci), a3 = __ldg(c3 + ci);
        const float lpc = lPc1[pi], lpp = lPp1[pi];
        addE += a3 * (lpc - w * lam);
        lPc0[pi] = w * (1.f - a1) * lam + a1 * lpc + lpp;
        lPp0[pi] = a2 * (lpc - w * lam);
        if (grad) {
            const float pc = __ldg(Pc + pi), pp = __ldg(Pp + pi);
            dsum += pc - (a1 * pc + a2 * pp + a3 * e);
        }
    }
    lamE_out[idx] += addE;
    if (grad) {
        const float gv = lam * dsum / (d * d);
        if (n_eps == 3) grad[comp * N + c] += gv;
        else atomicAdd(grad + c, gv);  // the three components of one cell share an isotropic entry
    }
}

}  // namespace fdtd
