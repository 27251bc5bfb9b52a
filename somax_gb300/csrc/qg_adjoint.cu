// Hand-written adjoint (vector-Jacobian product) of the fused RHS and of the PV inversion.
//
// Masked members (land mask): q is read as 0 on land, psi is 0 there and dq = 0 there (wind
// included), lap(q) is zero on land as on the ring; so the cotangent a, qb, psi and M Lf(a)
// are zeroed on land, and so are the cotangents of q and psi at land cells.  The masked
// inversion (two DST solves around the capacitance correction, psi = G x - G E C^-1 R G x with
// G the symmetric solve, C = R G E and R / E the restriction to / extension from the land
// boundary points) is a symmetric map, so the adjoint solve is the same masked inversion.
//
// Forward, per member (baroclinic.py:135-190; B is the optional ring zeroing of q, Z the
// zeroing of the psi ring of the baroclinic model, nu4 the biharmonic extension):
//   qb  = B q,   psi = Z Cm2l L^-1 Cl2m qb
//   dq  = -J(psi, qb) - J(psi, beta y) + nu lap(qb) - nu4 lap(lap qb)
//         + [l = 0] tau0 F / H0 - [l = nl-1] kappa lap(psi)             (J, lap: interior)
// The ring of dq holds the wind term only, so with a = the cotangent g masked to the interior:
//   qb_bar  = -Jg^T(psi; a) + nu Lf(a) - nu4 Lf(M Lf(a))
//   psi_bar = -Jf^T(qb; a) - Jb^T(a) - [l = nl-1] kappa Lf(a)
//   qb_bar += Cl2m^T L^-1 Cm2l^T Z psi_bar
//   q_bar   = B qb_bar
// Jg^T / Jf^T are the transposes of the Arakawa stencil in its second / first argument: for
// every stencil offset o of one argument, the cell b receives a(b - o) times the coefficient
// of that offset at b - o, a sum over the other argument around b - o.  Lf is the 5-point
// Laplacian over the whole array with zeros outside it (the transpose of the interior-only
// Laplacian applied to an interior-masked field) and M masks to the interior.  L^-1 is the
// DST-I solve: S is symmetric and the spectral divide diagonal, so it is self-adjoint and the
// same GEMM passes run it.  The parameter cotangents are the sums of g against the forward
// terms that are linear in nu, kappa, tau0 and nu4.
#include <cuda_bf16.h>

#include <algorithm>

#include "qg_internal.cuh"

namespace qg {

namespace {

constexpr int TX = 32, TY = 8, HB = 2;  // sub-tile and halo (the biharmonic reaches two cells)
constexpr int SX = TX + 2 * HB, SY = TY + 2 * HB;
constexpr int NT = 256;

__device__ __forceinline__ bool on_ring(int j, int i, int Ny, int Nx) {
    return j == 0 || i == 0 || j == Ny - 1 || i == Nx - 1;
}
__device__ __forceinline__ bool interior(int j, int i, int Ny, int Nx) {
    return j > 0 && i > 0 && j < Ny - 1 && i < Nx - 1;
}
__device__ __forceinline__ int64_t cidx(const MemberDev& M, int l, int j, int i) {
    return M.off_state + ((int64_t)l * M.Ny + j) * M.Nx + i;
}
__device__ __forceinline__ int64_t xidx(const MemberDev& M, int l, int j, int i) {
    return M.off_x + ((int64_t)l * M.Ny + j) * M.Px + i;
}

template <typename T>
__device__ __forceinline__ T warp_sum(T v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

}  // namespace

// Stencil part of the RHS VJP, one layer of one tile per block (grid: tiles x layers).
// Writes the direct cotangent of qb (x-row plane `direct`), accumulates Cm2l^T Z psi_bar into
// the FP32 modal plane `rhs` (atomics over the layers of a cell; zeroed by the caller) and the
// parameter cotangents into `pacc` (double, QG_NPARAMS per member).
__global__ void __launch_bounds__(NT) k_vjp_stencil(const MemberDev* __restrict__ members,
                                                    const StencilTile* __restrict__ tiles, int TXr, int TYr,
                                                    const float* __restrict__ q, int apply_bc,
                                                    const float* __restrict__ psi,
                                                    const float* __restrict__ gbar,
                                                    const float* __restrict__ params, float* __restrict__ direct,
                                                    float* __restrict__ rhs, double* __restrict__ pacc) {
    __shared__ float sa[SY][SX];  // a = interior-masked cotangent
    __shared__ float sq[SY][SX];  // qb
    __shared__ float sp[SY][SX];  // psi (layer, ring zeroed for the baroclinic model)
    __shared__ float sm[SY][SX];  // M Lf(a)
    __shared__ double red[3][NT / 32];
    const StencilTile t = tiles[blockIdx.x];
    const int l = blockIdx.y;
    const MemberDev& M = members[t.member];
    if (l >= M.nl) return;
    const int Ny = M.Ny, Nx = M.Nx, nl = M.nl;
    const float* P = params + (int64_t)t.member * QG_NPARAMS;
    const float nu = P[QG_P_NU], kappa = P[QG_P_KAPPA], nu4 = P[QG_P_NU4];
    const float idx2 = M.inv_dx2, idy2 = M.inv_dy2;
    const bool zero_psi_ring = !M.barotropic;
    for (int oy = 0; oy < TYr; oy += TY)
        for (int ox = 0; ox < TXr; ox += TX) {
            const int j0 = t.ty * TYr + oy - HB, i0 = t.tx * TXr + ox - HB;
            __syncthreads();
            for (int c = threadIdx.x; c < SY * SX; c += NT) {
                const int y = c / SX, x = c % SX, j = j0 + y, i = i0 + x;
                const bool in = j >= 0 && j < Ny && i >= 0 && i < Nx;
                // land of a masked member: dq = 0 there, q is read as 0 and psi is 0
                const bool land = in && is_land(M.mask, Ny, Nx, j, i);
                sa[y][x] = (in && interior(j, i, Ny, Nx) && !land) ? gbar[cidx(M, l, j, i)] : 0.f;
                sq[y][x] = (in && !(apply_bc && on_ring(j, i, Ny, Nx)) && !land) ? q[cidx(M, l, j, i)] : 0.f;
                sp[y][x] = (in && !land) ? psi[cidx(M, l, j, i)] : 0.f;
            }
            __syncthreads();
            for (int c = threadIdx.x; c < SY * SX; c += NT) {
                const int y = c / SX, x = c % SX, j = j0 + y, i = i0 + x;
                float v = 0.f;  // lap(qb) is zero on the ring and on land
                if (y > 0 && x > 0 && y < SY - 1 && x < SX - 1 && interior(j, i, Ny, Nx) &&
                    !is_land(M.mask, Ny, Nx, j, i))
                    v = (sa[y][x + 1] - 2.f * sa[y][x] + sa[y][x - 1]) * idx2 +
                        (sa[y + 1][x] - 2.f * sa[y][x] + sa[y - 1][x]) * idy2;
                sm[y][x] = v;
            }
            __syncthreads();
            double acc_nu = 0.0, acc_kappa = 0.0, acc_nu4 = 0.0;
            for (int c = threadIdx.x; c < TY * TX; c += NT) {
                const int y = c / TX + HB, x = c % TX + HB;
                const int j = j0 + y, i = i0 + x;
                if (j >= Ny || i >= Nx || oy + y - HB >= TYr || ox + x - HB >= TXr) continue;
                // A(dj, di): a at b + d;  F / G(cj, ci, dj, di): psi / qb at b + c + d
                auto A = [&](int dj, int di) { return sa[y + dj][x + di]; };
                auto F = [&](int cj, int ci, int dj, int di) { return sp[y + cj + dj][x + ci + di]; };
                auto G = [&](int cj, int ci, int dj, int di) { return sq[y + cj + dj][x + ci + di]; };
                // Jg^T: q at offset o of cell c = b - o; coefficient (in psi) of that offset at c
                const float jg =
                    A(-1, 0) * ((F(-1, 0, 0, 1) - F(-1, 0, 0, -1)) + (F(-1, 0, 1, 1) - F(-1, 0, 1, -1)))     // N
                    - A(1, 0) * ((F(1, 0, 0, 1) - F(1, 0, 0, -1)) + (F(1, 0, -1, 1) - F(1, 0, -1, -1)))      // S
                    - A(0, -1) * ((F(0, -1, 1, 0) - F(0, -1, -1, 0)) + (F(0, -1, 1, 1) - F(0, -1, -1, 1)))   // E
                    + A(0, 1) * ((F(0, 1, 1, 0) - F(0, 1, -1, 0)) + (F(0, 1, 1, -1) - F(0, 1, -1, -1)))      // W
                    + A(-1, -1) * (F(-1, -1, 0, 1) - F(-1, -1, 1, 0))                                        // NE
                    + A(1, -1) * (F(1, -1, -1, 0) - F(1, -1, 0, 1))                                          // SE
                    + A(-1, 1) * (F(-1, 1, 1, 0) - F(-1, 1, 0, -1))                                          // NW
                    + A(1, 1) * (F(1, 1, 0, -1) - F(1, 1, -1, 0));                                           // SW
                // Jf^T: psi at offset o of cell c = b - o; coefficient (in qb) of that offset at c
                const float jf =
                    A(0, -1) * ((G(0, -1, 1, 0) - G(0, -1, -1, 0)) + (G(0, -1, 1, 1) - G(0, -1, -1, 1)))     // E
                    - A(0, 1) * ((G(0, 1, 1, 0) - G(0, 1, -1, 0)) + (G(0, 1, 1, -1) - G(0, 1, -1, -1)))      // W
                    - A(-1, 0) * ((G(-1, 0, 0, 1) - G(-1, 0, 0, -1)) + (G(-1, 0, 1, 1) - G(-1, 0, 1, -1)))   // N
                    + A(1, 0) * ((G(1, 0, 0, 1) - G(1, 0, 0, -1)) + (G(1, 0, -1, 1) - G(1, 0, -1, -1)))      // S
                    + A(-1, -1) * (G(-1, -1, 1, 0) - G(-1, -1, 0, 1))                                        // NE
                    + A(-1, 1) * (G(-1, 1, 0, -1) - G(-1, 1, 1, 0))                                          // NW
                    + A(1, -1) * (G(1, -1, 0, 1) - G(1, -1, -1, 0))                                          // SE
                    + A(1, 1) * (G(1, 1, -1, 0) - G(1, 1, 0, -1));                                           // SW
                // J(psi, beta y) = beta / (12 dx) [4 (fE - fW) + fNE - fNW + fSE - fSW]
                const float jb = 4.f * (A(0, -1) - A(0, 1)) + (A(-1, -1) - A(-1, 1)) + (A(1, -1) - A(1, 1));
                const float lfa =
                    (A(0, 1) - 2.f * A(0, 0) + A(0, -1)) * idx2 + (A(1, 0) - 2.f * A(0, 0) + A(-1, 0)) * idy2;
                const float lfm = (sm[y][x + 1] - 2.f * sm[y][x] + sm[y][x - 1]) * idx2 +
                                  (sm[y + 1][x] - 2.f * sm[y][x] + sm[y - 1][x]) * idy2;
                const bool land_b = is_land(M.mask, Ny, Nx, j, i);  // q and psi of land cells are fixed at 0
                direct[xidx(M, l, j, i)] = land_b ? 0.f : -jg * M.inv_12dxdy + nu * lfa - nu4 * lfm;
                float pb = -jf * M.inv_12dxdy - jb * M.beta_12dx;
                if (l == nl - 1) pb -= kappa * lfa;
                if (!(zero_psi_ring && on_ring(j, i, Ny, Nx)) && !land_b)
                    for (int m = 0; m < nl; ++m) atomicAdd(&rhs[xidx(M, m, j, i)], M.Cm2l[l * kMaxLayers + m] * pb);
                if (interior(j, i, Ny, Nx)) {
                    const float lq = (G(0, 0, 0, 1) - 2.f * G(0, 0, 0, 0) + G(0, 0, 0, -1)) * idx2 +
                                     (G(0, 0, 1, 0) - 2.f * G(0, 0, 0, 0) + G(0, 0, -1, 0)) * idy2;
                    acc_nu += (double)A(0, 0) * lq;
                    acc_nu4 -= (double)sm[y][x] * lq;  // -<a, lap(M lap qb)> = -<M Lf(a), lap qb>
                    if (l == nl - 1) {
                        const float lp = (F(0, 0, 0, 1) - 2.f * F(0, 0, 0, 0) + F(0, 0, 0, -1)) * idx2 +
                                         (F(0, 0, 1, 0) - 2.f * F(0, 0, 0, 0) + F(0, 0, -1, 0)) * idy2;
                        acc_kappa -= (double)A(0, 0) * lp;
                    }
                }
            }
            acc_nu = warp_sum(acc_nu);
            acc_kappa = warp_sum(acc_kappa);
            acc_nu4 = warp_sum(acc_nu4);
            const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
            if (lane == 0) {
                red[0][w] = acc_nu;
                red[1][w] = acc_kappa;
                red[2][w] = acc_nu4;
            }
            __syncthreads();
            if (threadIdx.x == 0) {
                double s0 = 0, s1 = 0, s2 = 0;
                for (int k = 0; k < NT / 32; ++k) {
                    s0 += red[0][k];
                    s1 += red[1][k];
                    s2 += red[2][k];
                }
                atomicAdd(&pacc[QG_NPARAMS * t.member + QG_P_NU], s0);
                atomicAdd(&pacc[QG_NPARAMS * t.member + QG_P_KAPPA], s1);
                atomicAdd(&pacc[QG_NPARAMS * t.member + QG_P_NU4], s2);
            }
        }
}

// tau0 cotangent: the sum over every cell of layer 0 (ring included) of g F / H0.
__global__ void __launch_bounds__(NT) k_vjp_tau(const MemberDev* __restrict__ members, int n_members,
                                                const float* __restrict__ gbar, double* __restrict__ pacc) {
    __shared__ double red[NT / 32];
    const int mem = blockIdx.y;
    if (mem >= n_members) return;
    const MemberDev& M = members[mem];
    double acc = 0.0;
    const int64_t n = (int64_t)M.Ny * M.Nx;
    for (int64_t c = blockIdx.x * (int64_t)NT + threadIdx.x; c < n; c += (int64_t)gridDim.x * NT) {
        const int j = (int)(c / M.Nx), i = (int)(c % M.Nx);
        if (is_land(M.mask, M.Ny, M.Nx, j, i)) continue;  // dq = 0 on land, wind included
        acc += (double)gbar[cidx(M, 0, j, i)] * M.F[j] * M.invH0;
    }
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0;
        for (int k = 0; k < NT / 32; ++k) s += red[k];
        atomicAdd(&pacc[QG_NPARAMS * mem + QG_P_TAU0], s);
    }
}

// Right-hand side of the adjoint solve in the GEMM operand format (plus its FP32 copy for the
// refinement residual).  From the FP32 modal plane `rhs` when `psi_bar` is null, else
// Cm2l^T Z psi_bar of a caller-packed layer cotangent (the VJP of the inversion).
__global__ void __launch_bounds__(NT) k_vjp_operand(const MemberDev* __restrict__ members,
                                                    const StencilTile* __restrict__ tiles, int TXr, int TYr,
                                                    const float* __restrict__ rhs,
                                                    const float* __restrict__ psi_bar, void* xa, int xa_fmt,
                                                    float* xq, int64_t xplane) {
    const StencilTile t = tiles[blockIdx.x];
    const MemberDev& M = members[t.member];
    const int nl = M.nl;
    for (int c = threadIdx.x; c < TXr * TYr; c += NT) {
        const int j = t.ty * TYr + c / TXr, i = t.tx * TXr + c % TXr;
        if (j >= M.Ny || i >= M.Nx) continue;
        float pb[kMaxLayers];
        if (psi_bar) {
            const bool zero = (!M.barotropic && on_ring(j, i, M.Ny, M.Nx)) || is_land(M.mask, M.Ny, M.Nx, j, i);
            for (int l = 0; l < nl; ++l) pb[l] = zero ? 0.f : psi_bar[cidx(M, l, j, i)];
        }
        for (int m = 0; m < nl; ++m) {
            const int64_t o = xidx(M, m, j, i);
            float v = 0.f;
            if (psi_bar) {
                for (int l = 0; l < nl; ++l) v = fmaf(M.Cm2l[l * kMaxLayers + m], pb[l], v);
            } else {
                v = rhs[o];
            }
            if (xa_fmt == FMT_F32) {
                static_cast<float*>(xa)[o] = v;
            } else {
                __nv_bfloat16* p = static_cast<__nv_bfloat16*>(xa);
                const __nv_bfloat16 hi = __float2bfloat16_rn(v);
                p[o] = hi;
                p[xplane + o] = __float2bfloat16_rn(v - __bfloat162float(hi));
            }
            if (xq) xq[o] = v;
        }
    }
}

// q_bar = B (direct + Cl2m^T x_bar) in caller packing, x_bar the adjoint solve's output.
__global__ void __launch_bounds__(NT) k_vjp_finish(const MemberDev* __restrict__ members,
                                                   const StencilTile* __restrict__ tiles, int TXr, int TYr,
                                                   const float* __restrict__ direct,
                                                   const float* __restrict__ xbar, int apply_bc,
                                                   float* __restrict__ qbar) {
    const StencilTile t = tiles[blockIdx.x];
    const MemberDev& M = members[t.member];
    const int nl = M.nl;
    for (int c = threadIdx.x; c < TXr * TYr; c += NT) {
        const int j = t.ty * TYr + c / TXr, i = t.tx * TXr + c % TXr;
        if (j >= M.Ny || i >= M.Nx) continue;
        // q of the ring (under the BC) and of land cells is not read by the forward
        const bool zero = (apply_bc && on_ring(j, i, M.Ny, M.Nx)) || is_land(M.mask, M.Ny, M.Nx, j, i);
        float xb[kMaxLayers];
        for (int m = 0; m < nl; ++m) xb[m] = xbar[xidx(M, m, j, i)];
        for (int l = 0; l < nl; ++l) {
            float v = direct ? direct[xidx(M, l, j, i)] : 0.f;
            for (int m = 0; m < nl; ++m) v = fmaf(M.Cl2m[m * kMaxLayers + l], xb[m], v);
            qbar[cidx(M, l, j, i)] = zero ? 0.f : v;
        }
    }
}

__global__ void k_vjp_params(const double* __restrict__ pacc, int n, float* __restrict__ pbar) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k < n) pbar[k] = (float)pacc[k];
}

cudaError_t launch_vjp_stencil(const VjpArgs& v, cudaStream_t s) {
    k_vjp_stencil<<<dim3(v.ntiles, v.max_nl), NT, 0, s>>>(v.members, v.tiles, v.tile_x, v.tile_y, v.q, v.apply_bc,
                                                          v.psi, v.gbar, v.params, v.direct, v.rhs, v.pacc);
    cudaError_t e = cudaGetLastError();
    if (!e) {
        k_vjp_tau<<<dim3(16, v.n_members), NT, 0, s>>>(v.members, v.n_members, v.gbar, v.pacc);
        e = cudaGetLastError();
    }
    return e;
}

cudaError_t launch_vjp_operand(const VjpArgs& v, const float* psi_bar, cudaStream_t s) {
    k_vjp_operand<<<v.ntiles, NT, 0, s>>>(v.members, v.tiles, v.tile_x, v.tile_y, v.rhs, psi_bar, v.xa, v.xa_fmt,
                                          v.xq, v.xplane);
    return cudaGetLastError();
}

cudaError_t launch_vjp_finish(const VjpArgs& v, const float* xbar, float* qbar, float* pbar, cudaStream_t s) {
    k_vjp_finish<<<v.ntiles, NT, 0, s>>>(v.members, v.tiles, v.tile_x, v.tile_y, v.direct, xbar, v.apply_bc, qbar);
    cudaError_t e = cudaGetLastError();
    if (!e && pbar) {
        const int n = v.n_members * QG_NPARAMS;
        k_vjp_params<<<(n + 127) / 128, 128, 0, s>>>(v.pacc, n, pbar);
        e = cudaGetLastError();
    }
    return e;
}

// Linear combinations over packed fields (caller packing, n floats each) for the Runge-Kutta
// step's adjoint: out = base + sum_j c_j x_j (stage inputs), and the reverse sweep's
// scatter of one stage cotangent Ybar: y_bar += Ybar, kbar_j += c_j Ybar.
struct LinComb {
    const float* x[kMaxButcher];
    float* y[kMaxButcher];
    float c[kMaxButcher];
    int n_terms;
};

__global__ void k_lincomb(float* __restrict__ out, const float* __restrict__ base, LinComb lc, int64_t n) {
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += nth) {
        float v = base[t];
        for (int j = 0; j < lc.n_terms; ++j) v = fmaf(lc.c[j], lc.x[j][t], v);
        out[t] = v;
    }
}

// y_bar += Ybar and kbar_j += c_j Ybar (j < n_terms), in one pass over Ybar.
__global__ void k_scatter_bar(float* __restrict__ ybar, const float* __restrict__ Yb, LinComb lc, int64_t n) {
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += nth) {
        const float v = Yb[t];
        ybar[t] += v;
        for (int j = 0; j < lc.n_terms; ++j) lc.y[j][t] = fmaf(lc.c[j], v, lc.y[j][t]);
    }
}

// kbar_s = c_s g for every stage s (the cotangents of the stage derivatives at the step's end).
__global__ void k_fanout(const float* __restrict__ g, LinComb lc, int64_t n) {
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += nth) {
        const float v = g[t];
        for (int j = 0; j < lc.n_terms; ++j) lc.y[j][t] = lc.c[j] * v;
    }
}

namespace {
int lincomb_grid(int64_t n) { return (int)std::min<int64_t>(8192, std::max<int64_t>(1, (n + 255) / 256)); }
}  // namespace

cudaError_t launch_lincomb(float* out, const float* base, const float* const* x, const float* c, int n_terms,
                           int64_t n, cudaStream_t s) {
    LinComb lc{};
    lc.n_terms = n_terms;
    for (int j = 0; j < n_terms; ++j) {
        lc.x[j] = x[j];
        lc.c[j] = c[j];
    }
    k_lincomb<<<lincomb_grid(n), 256, 0, s>>>(out, base, lc, n);
    return cudaGetLastError();
}

cudaError_t launch_scatter_bar(float* ybar, const float* Yb, float* const* kbar, const float* c, int n_terms,
                               int64_t n, cudaStream_t s) {
    LinComb lc{};
    lc.n_terms = n_terms;
    for (int j = 0; j < n_terms; ++j) {
        lc.y[j] = kbar[j];
        lc.c[j] = c[j];
    }
    k_scatter_bar<<<lincomb_grid(n), 256, 0, s>>>(ybar, Yb, lc, n);
    return cudaGetLastError();
}

cudaError_t launch_fanout(const float* g, float* const* out, const float* c, int n_terms, int64_t n, cudaStream_t s) {
    LinComb lc{};
    lc.n_terms = n_terms;
    for (int j = 0; j < n_terms; ++j) {
        lc.y[j] = out[j];
        lc.c[j] = c[j];
    }
    k_fanout<<<lincomb_grid(n), 256, 0, s>>>(g, lc, n);
    return cudaGetLastError();
}

cudaError_t launch_vjp_params_only(const VjpArgs& v, float* pbar, cudaStream_t s) {
    const int n = v.n_members * QG_NPARAMS;
    k_vjp_params<<<(n + 127) / 128, 128, 0, s>>>(v.pacc, n, pbar);
    return cudaGetLastError();
}

}  // namespace qg
