// Full 3x3 anisotropic half-steps (sm_103a): the tensor branch of update_E / update_H and of
// their reverse (fdtdx/fdtd/update.py:356-492, 751-807, 641-676, 956-995) with the update
// matrices and the four-point averages of fdtdx/fdtd/misc.py:69-213.
//
// A component's update reads the other two components of the updated field and of the curl
// on a four-cell stencil around its own Yee location, so one half-step is two passes over the
// grid: the curl (with its CPML terms; psi advanced in a forward step, frozen in a reverse
// one) into a scratch field K, with a copy of the updated field into a second scratch T when
// the update is in place, then the tensor update from K and T.  Complex (Bloch) fields run
// both passes part by part (each pass over both parts before the next pass starts, since a
// wrapped neighbour mixes the parts); K and T hold the parts planar like the fields.
#pragma once
#include "fdtd_kernels.cuh"

namespace fdtd {

// Pass 1: K = the curl of the differentiated field at every cell, CPML terms included, and
// T = the updated field's values (when T is given: an in-place update).
template <bool REV, bool HSIDE>
__global__ void __launch_bounds__(256) k_full_curl(const __grid_constant__ UpdArgs a, float* __restrict__ K,
                                                   float* __restrict__ T) {
    const Geo& g = a.g;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.N) return;
    const int k = (int)(c % g.nz);
    const long long r = c / g.nz;
    const int j = (int)(r % g.ny);
    const int i = (int)(r / g.ny);
    const long long N = g.N;
    const float* __restrict__ F = a.F;
    const float fx = __ldg(F + c), fy = __ldg(F + N + c), fz = __ldg(F + 2 * N + c);
    float d[6];
    if (!HSIDE) {  // backward differences of H (curl_H, fdtdx/core/physics/curl.py:314-397)
        d[0] = fz - ld_halo(g, F, 2, i, j - 1, k);
        d[1] = fy - ld_halo(g, F, 1, i, j, k - 1);
        d[2] = fx - ld_halo(g, F, 0, i, j, k - 1);
        d[3] = fz - ld_halo(g, F, 2, i - 1, j, k);
        d[4] = fy - ld_halo(g, F, 1, i - 1, j, k);
        d[5] = fx - ld_halo(g, F, 0, i, j - 1, k);
    } else {       // forward differences of E (curl_E, curl.py:227-311)
        d[0] = ld_halo(g, F, 2, i, j + 1, k) - fz;
        d[1] = ld_halo(g, F, 1, i, j, k + 1) - fy;
        d[2] = ld_halo(g, F, 0, i, j, k + 1) - fx;
        d[3] = ld_halo(g, F, 2, i + 1, j, k) - fz;
        d[4] = ld_halo(g, F, 1, i + 1, j, k) - fy;
        d[5] = ld_halo(g, F, 0, i, j + 1, k) - fx;
    }
    float cu[3] = {d[0] - d[1], d[2] - d[3], d[4] - d[5]};
    if (a.n_slab) {
        PsiPre pr;
        psi_fetch(a, i, j, k, pr);
        cpml_apply<REV, HSIDE>(a, i, j, k, d, cu, pr);
    }
#pragma unroll
    for (int q = 0; q < 3; ++q) K[q * N + c] = cu[q];
    if (T) {
#pragma unroll
        for (int q = 0; q < 3; ++q) T[q * N + c] = __ldg(a.Uin + q * N + c);
    }
}

// Component `comp` of a field averaged onto the Yee location of component `loc`: the E-type
// stencil (fdtdx/fdtd/misc.py:132-171) over x, x + e_loc, x - e_comp, x + e_loc - e_comp; the
// H-type one (misc.py:174-213) with both offsets negated.
template <bool HSIDE>
__device__ __forceinline__ float avg_onto(const Geo& g, const float* __restrict__ f, int comp, int loc, int i, int j,
                                          int k) {
    const int sl = HSIDE ? -1 : 1, sc = HSIDE ? 1 : -1;
    const int li = loc == 0 ? sl : 0, lj = loc == 1 ? sl : 0, lk = loc == 2 ? sl : 0;
    const int ci = comp == 0 ? sc : 0, cj = comp == 1 ? sc : 0, ck = comp == 2 ? sc : 0;
    const float s = ld_halo(g, f, comp, i, j, k) + ld_halo(g, f, comp, i + li, j + lj, k + lk);
    const float t = ld_halo(g, f, comp, i + ci, j + cj, k + ck) + ld_halo(g, f, comp, i + li + ci, j + lj + cj, k + lk + ck);
    return (s + t) / 4.f;
}

// Pass 2: F_i = sum_j A_ij F_j@i + s sum_j B_ij K_j@i (update.py:474-492, 791-807), with
// forward A = M1^-1 M2 = 2 M1^-1 - I and B = c M1^-1 inv, reverse A = M2^-1 M1 = 2 M2^-1 - I
// and B = c M2^-1 inv, M1,2 = I +- (c eta / 2) inv sigma (eta = eta0 for E, 1 / eta0 for H;
// misc.py:69-129); without conductivity A = I and B = c inv.  s = +1 for the forward E and
// the reverse H update, -1 for the other two.  Diagonal terms are local, off-diagonal ones
// averaged onto the row's location; conductor faces are zeroed afterwards.
template <bool REV, bool HSIDE>
__global__ void __launch_bounds__(256) k_full_apply(const __grid_constant__ UpdArgs a, const float* __restrict__ K,
                                                    const float* __restrict__ Fo) {
    const Geo& g = a.g;
    const long long c = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= g.N) return;
    const int k = (int)(c % g.nz);
    const long long r = c / g.nz;
    const int j = (int)(r % g.ny);
    const int i = (int)(r / g.ny);
    const long long N = g.N;
    float inv[9], A[9], B[9];
    tensor_at(a.mat, a.n_mat, a.mat_scalar, N, c, inv);
    if (a.sig) {
        float sg[9], M[9], Mi[9];
        tensor_at(a.sig, a.n_sig, 0.f, N, c, sg);
        const float kq = HSIDE ? g.c / g.eta0 / 2.f : g.c * g.eta0 / 2.f;
#pragma unroll
        for (int row = 0; row < 3; ++row)
#pragma unroll
            for (int col = 0; col < 3; ++col) {
                const float pc = inv[row * 3] * sg[col] + inv[row * 3 + 1] * sg[3 + col] + inv[row * 3 + 2] * sg[6 + col];
                M[row * 3 + col] = (row == col ? 1.f : 0.f) + (REV ? -kq : kq) * pc;
            }
        inverse3(M, Mi);
#pragma unroll
        for (int row = 0; row < 3; ++row)
#pragma unroll
            for (int col = 0; col < 3; ++col) {
                A[row * 3 + col] = 2.f * Mi[row * 3 + col] - (row == col ? 1.f : 0.f);
                B[row * 3 + col] = g.c * (Mi[row * 3] * inv[col] + Mi[row * 3 + 1] * inv[3 + col] + Mi[row * 3 + 2] * inv[6 + col]);
            }
    } else {
#pragma unroll
        for (int q = 0; q < 9; ++q) {
            A[q] = (q % 4 == 0) ? 1.f : 0.f;
            B[q] = g.c * inv[q];
        }
    }
    const float s = (HSIDE != REV) ? -1.f : 1.f;
    const int wall = HSIDE ? g.pmc : g.pec;
#pragma unroll
    for (int row = 0; row < 3; ++row) {
        float acc_a = A[row * 4] * __ldg(Fo + row * N + c);
        float acc_b = B[row * 4] * __ldg(K + row * N + c);
#pragma unroll
        for (int col = 0; col < 3; ++col) {
            if (col == row) continue;
            const float ac = A[row * 3 + col], bc = B[row * 3 + col];
            if (ac != 0.f) acc_a += ac * avg_onto<HSIDE>(g, Fo, col, row, i, j, k);
            if (bc != 0.f) acc_b += bc * avg_onto<HSIDE>(g, K, col, row, i, j, k);
        }
        float u = acc_a + s * acc_b;
        if (wall && face_zero(g, wall, row, i, j, k)) u = 0.f;
        a.Uout[row * N + c] = u;
    }
}

}  // namespace fdtd
