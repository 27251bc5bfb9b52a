// Memory-bound kernels of the QG time step: the fused RHS stencil (with the RK stage update
// and the next stage's layer->mode prologue fused in), the layer->mode prologue on its own,
// the mode->layer epilogue, the Helmholtz residual and the diagnostics.
//
// Every kernel walks a list of 2-D tiles (StencilTile) that may belong to different members
// of an ensemble; a block owns one tile and all layers of it.
#include <cuda_bf16.h>

#include "qg_internal.cuh"

namespace qg {

namespace {

constexpr int TX = kStencilTX;  // tile width  (x)
constexpr int TY = kStencilTY;  // tile height (y)
constexpr int HALO = 2;         // biharmonic needs two cells
constexpr int SW = TX + 2 * HALO;
constexpr int SH = TY + 2 * HALO;
constexpr int NTHREADS = 256;

// Copy a member's constants into shared memory (one 4-byte word per thread per pass).
__device__ __forceinline__ void load_member(MemberDev* dst, const MemberDev* src) {
    const int* s = reinterpret_cast<const int*>(src);
    int* d = reinterpret_cast<int*>(dst);
    for (int w = threadIdx.x; w < (int)(sizeof(MemberDev) / 4); w += blockDim.x) d[w] = s[w];
}

__device__ __forceinline__ bool on_ring(int j, int i, int Ny, int Nx) {
    return j == 0 || i == 0 || j == Ny - 1 || i == Nx - 1;
}

// Index of (l, j, i) in a packed field.
__device__ __forceinline__ int64_t caller_idx(const MemberDev& M, int l, int j, int i) {
    return M.off_state + ((int64_t)l * M.Ny + j) * M.Nx + i;
}
__device__ __forceinline__ int64_t xrow_idx(const MemberDev& M, int l, int j, int i) {
    return M.off_x + ((int64_t)l * M.Ny + j) * M.Px + i;
}

__device__ __forceinline__ void store_plane(void* base, int fmt, int64_t plane_elems, int64_t idx,
                                            float v) {
    if (fmt == FMT_F32) {
        static_cast<float*>(base)[idx] = v;
    } else {
        __nv_bfloat16 hi = __float2bfloat16_rn(v);
        __nv_bfloat16 lo = __float2bfloat16_rn(v - __bfloat162float(hi));
        __nv_bfloat16* p = static_cast<__nv_bfloat16*>(base);
        p[idx] = hi;
        p[plane_elems + idx] = lo;
    }
}

}  // namespace

// ---------------------------------------------------------------------------------------
// Layer -> mode prologue: xa = Cl2m * BC(q) for every cell of every member.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_prep(const MemberDev* __restrict__ members,
                                                   const StencilTile* __restrict__ tiles,
                                                   const float* __restrict__ q, float* q_inplace,
                                                   int apply_bc, void* xa, int xa_fmt,
                                                   float* xq, int64_t xplane) {
    __shared__ MemberDev M;
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    const int nl = M.nl;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        const bool ring = on_ring(j, i, M.Ny, M.Nx);
        float v[kMaxLayers];
        for (int l = 0; l < nl; ++l) {
            v[l] = (apply_bc && ring) ? 0.f : q[caller_idx(M, l, j, i)];
            if (q_inplace && apply_bc && ring) q_inplace[caller_idx(M, l, j, i)] = 0.f;
        }
        for (int m = 0; m < nl; ++m) {
            float s = 0.f;
            for (int l = 0; l < nl; ++l) s = fmaf(M.Cl2m[m * kMaxLayers + l], v[l], s);
            store_plane(xa, xa_fmt, xplane, xrow_idx(M, m, j, i), s);
            if (xq) xq[xrow_idx(M, m, j, i)] = s;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Fused RHS stencil.  Per cell and layer (baroclinic.py:161-190, barotropic.py:123-152):
//   dq = -J(psi, q + beta y) + [l = 0] tau0 F / H0 - [l = nl-1] kappa lap(psi) + nu lap(q)
//        - nu4 lap(lap q)                                   (biharmonic extension)
// with psi = Cm2l psi_hat (ring zeroed for the baroclinic model).  J(psi, beta y) is
// evaluated in closed form for the linear beta y (exact for the Arakawa stencil), which
// keeps FP32 from losing q against the much larger beta y.  On the ring dq is the wind
// term only (J and the Laplacians are interior-only there).
// Step mode fuses the Shu-Osher stage update y_next = a y0 + b (y_s + dt dq) and the next
// stage's layer->mode prologue.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_stencil(StencilArgs a, int64_t xplane) {
    extern __shared__ float smem[];
    __shared__ MemberDev M;
    const StencilTile t = a.tiles[blockIdx.x];
    load_member(&M, a.members + t.member);
    __syncthreads();

    const int nl = M.nl, Ny = M.Ny, Nx = M.Nx;
    const float* P = a.params + (int64_t)t.member * QG_NPARAMS;
    const float nu = P[QG_P_NU], kappa = P[QG_P_KAPPA], tau0 = P[QG_P_TAU0], nu4 = P[QG_P_NU4];

    float* sq = smem;                // nl x SH x SW : q (BC applied on read)
    float* sp = sq + nl * SH * SW;   // nl x SH x SW : psi (layer space)
    float* sl = sp + nl * SH * SW;   // nl x SH x SW : lap(q), only when nu4 != 0

    const int j0 = t.ty * TY - HALO, i0 = t.tx * TX - HALO;
    for (int c = threadIdx.x; c < SH * SW; c += blockDim.x) {
        const int sy = c / SW, sx = c % SW;
        const int j = j0 + sy, i = i0 + sx;
        const bool in = j >= 0 && j < Ny && i >= 0 && i < Nx;
        const bool ring = in && on_ring(j, i, Ny, Nx);
        float ph[kMaxLayers];
        for (int m = 0; m < nl; ++m) ph[m] = in ? a.psi_hat[xrow_idx(M, m, j, i)] : 0.f;
        for (int l = 0; l < nl; ++l) {
            float qv = 0.f;
            if (in && !(a.apply_bc && ring))
                qv = a.q_internal ? a.q[xrow_idx(M, l, j, i)] : a.q[caller_idx(M, l, j, i)];
            sq[(l * SH + sy) * SW + sx] = qv;
            float p = 0.f;
            for (int m = 0; m < nl; ++m) p = fmaf(M.Cm2l[l * kMaxLayers + m], ph[m], p);
            if (!in || (ring && !M.barotropic)) p = 0.f;
            sp[(l * SH + sy) * SW + sx] = p;
        }
    }
    __syncthreads();

    const float idx2 = M.inv_dx2, idy2 = M.inv_dy2;
    if (nu4 != 0.f) {
        for (int c = threadIdx.x; c < SH * SW; c += blockDim.x) {
            const int sy = c / SW, sx = c % SW;
            const int j = j0 + sy, i = i0 + sx;
            const bool interior = j > 0 && j < Ny - 1 && i > 0 && i < Nx - 1 && sy > 0 &&
                                  sy < SH - 1 && sx > 0 && sx < SW - 1;
            for (int l = 0; l < nl; ++l) {
                const float* Q = sq + l * SH * SW;
                float v = 0.f;
                if (interior) {
                    const float ctr = Q[sy * SW + sx];
                    v = (Q[sy * SW + sx + 1] - 2.f * ctr + Q[sy * SW + sx - 1]) * idx2 +
                        (Q[(sy + 1) * SW + sx] - 2.f * ctr + Q[(sy - 1) * SW + sx]) * idy2;
                }
                sl[(l * SH + sy) * SW + sx] = v;
            }
        }
        __syncthreads();
    }

    bool bad = false;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int ly = c / TX, lx = c % TX;
        const int j = t.ty * TY + ly, i = t.tx * TX + lx;
        if (j >= Ny || i >= Nx) continue;
        const bool ring = on_ring(j, i, Ny, Nx);
        const int sy = ly + HALO, sx = lx + HALO;
        const float wind = tau0 * M.F[j] * M.invH0;
        float d[kMaxLayers];
        for (int l = 0; l < nl; ++l) {
            if (ring) {
                d[l] = (l == 0) ? wind : 0.f;
                continue;
            }
            const float* Q = sq + l * SH * SW;
            const float* S = sp + l * SH * SW;
            auto q_ = [&](int dj, int di) { return Q[(sy + dj) * SW + sx + di]; };
            auto p_ = [&](int dj, int di) { return S[(sy + dj) * SW + sx + di]; };
            const float fE = p_(0, 1), fW = p_(0, -1), fN = p_(1, 0), fS = p_(-1, 0);
            const float fNE = p_(1, 1), fNW = p_(1, -1), fSE = p_(-1, 1), fSW = p_(-1, -1);
            const float gE = q_(0, 1), gW = q_(0, -1), gN = q_(1, 0), gS = q_(-1, 0);
            const float gNE = q_(1, 1), gNW = q_(1, -1), gSE = q_(-1, 1), gSW = q_(-1, -1);
            const float jpp = (fE - fW) * (gN - gS) - (fN - fS) * (gE - gW);
            const float jpx = fE * (gNE - gSE) - fW * (gNW - gSW) - fN * (gNE - gNW) + fS * (gSE - gSW);
            const float jxp = gN * (fNE - fNW) - gS * (fSE - fSW) - gE * (fNE - fSE) + gW * (fNW - fSW);
            const float Jq = (jpp + jpx + jxp) * M.inv_12dxdy;
            const float Jb = (4.f * (fE - fW) + (fNE - fNW) + (fSE - fSW)) * M.beta_12dx;
            float v = -(Jq + Jb);
            if (l == 0) v += wind;
            if (l == nl - 1) {
                const float lp = (fE - 2.f * p_(0, 0) + fW) * idx2 + (fN - 2.f * p_(0, 0) + fS) * idy2;
                v += -kappa * lp;
            }
            const float lq = (gE - 2.f * q_(0, 0) + gW) * idx2 + (gN - 2.f * q_(0, 0) + gS) * idy2;
            v += nu * lq;
            if (nu4 != 0.f) {
                const float* L = sl + l * SH * SW;
                auto l_ = [&](int dj, int di) { return L[(sy + dj) * SW + sx + di]; };
                const float bl = (l_(0, 1) - 2.f * l_(0, 0) + l_(0, -1)) * idx2 +
                                 (l_(1, 0) - 2.f * l_(0, 0) + l_(-1, 0)) * idy2;
                v -= nu4 * bl;
            }
            d[l] = v;
        }
        for (int l = 0; l < nl; ++l) bad |= !isfinite(d[l]);

        if (a.dq) {
            for (int l = 0; l < nl; ++l) a.dq[caller_idx(M, l, j, i)] = d[l];
            continue;
        }
        // step mode
        float yn[kMaxLayers];
        for (int l = 0; l < nl; ++l) {
            const float y0 = a.y0[caller_idx(M, l, j, i)];
            if (ring) {
                // The ring tendency is state independent (wind only), so every consistent
                // RK scheme ends at y0 + dt * dq there; stage inputs carry a zero ring (BC).
                yn[l] = a.final_stage ? y0 + a.dt * d[l] : 0.f;
            } else {
                const float ys = sq[(l * SH + sy) * SW + sx];
                yn[l] = a.a * y0 + a.b * (ys + a.dt * d[l]);
            }
            bad |= !isfinite(yn[l]);
            const int64_t o = a.y_next_internal ? xrow_idx(M, l, j, i) : caller_idx(M, l, j, i);
            a.y_next[o] = yn[l];
        }
        if (a.xa) {
            for (int m = 0; m < nl; ++m) {
                float s = 0.f;
                if (!ring)
                    for (int l = 0; l < nl; ++l) s = fmaf(M.Cl2m[m * kMaxLayers + l], yn[l], s);
                store_plane(a.xa, a.xa_fmt, xplane, xrow_idx(M, m, j, i), s);
                if (a.xq) a.xq[xrow_idx(M, m, j, i)] = s;
            }
        }
    }
    if (bad && a.flags) atomicOr(a.flags, 1);
}

// ---------------------------------------------------------------------------------------
// Mode -> layer epilogue for qg_invert: psi = Cm2l psi_hat, ring zeroed (baroclinic).
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_mode_to_layer(const MemberDev* __restrict__ members,
                                                            const StencilTile* __restrict__ tiles,
                                                            const float* __restrict__ psi_hat,
                                                            float* __restrict__ psi) {
    __shared__ MemberDev M;
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    const int nl = M.nl;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        const bool zero = !M.barotropic && on_ring(j, i, M.Ny, M.Nx);
        float ph[kMaxLayers];
        for (int m = 0; m < nl; ++m) ph[m] = psi_hat[xrow_idx(M, m, j, i)];
        for (int l = 0; l < nl; ++l) {
            float p = 0.f;
            for (int m = 0; m < nl; ++m) p = fmaf(M.Cm2l[l * kMaxLayers + m], ph[m], p);
            psi[caller_idx(M, l, j, i)] = zero ? 0.f : p;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Helmholtz residual in modal space for one refinement sweep:
//   r_m = qm_m - (lap_full psi_hat_m - lam_m psi_hat_m)
// where lap_full is the full-array 5-point operator with zeros outside the array (the
// operator the DST-I solve inverts).  qm is the FP32 modal right-hand side.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_residual(const MemberDev* __restrict__ members,
                                                       const StencilTile* __restrict__ tiles,
                                                       const float* __restrict__ qm,
                                                       const float* __restrict__ psi_hat,
                                                       void* out, int out_fmt, int64_t xplane) {
    __shared__ MemberDev M;
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    const int nl = M.nl, Ny = M.Ny, Nx = M.Nx;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= Ny || i >= Nx) continue;
        for (int m = 0; m < nl; ++m) {
            auto P = [&](int jj, int ii) {
                return (jj < 0 || jj >= Ny || ii < 0 || ii >= Nx) ? 0.f : psi_hat[xrow_idx(M, m, jj, ii)];
            };
            const float c0 = P(j, i);
            const float lap = (P(j, i + 1) - 2.f * c0 + P(j, i - 1)) * M.inv_dx2 +
                              (P(j + 1, i) - 2.f * c0 + P(j - 1, i)) * M.inv_dy2;
            const float r = qm[xrow_idx(M, m, j, i)] - (lap - M.lam[m] * c0);
            store_plane(out, out_fmt, xplane, xrow_idx(M, m, j, i), r);
        }
    }
}

// ---------------------------------------------------------------------------------------
// Diagnostics (baroclinic.py:197-228): per layer KE = 1/2 sum_int (u_T^2 + v_T^2) dx dy,
// enstrophy = 1/2 sum_int q^2 dx dy, u = -d_y psi (V points), v = d_x psi (U points),
// both interior-written and averaged back to T points.  Sums accumulate in double.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_diag(const MemberDev* __restrict__ members,
                                                   const StencilTile* __restrict__ tiles,
                                                   const float* __restrict__ q,
                                                   const float* __restrict__ psi_hat,
                                                   double* __restrict__ acc) {
    __shared__ MemberDev M;
    __shared__ double red[2 * kMaxLayers][NTHREADS / 32];
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    const int nl = M.nl, Ny = M.Ny, Nx = M.Nx;
    double ke[kMaxLayers], en[kMaxLayers];
    for (int l = 0; l < nl; ++l) ke[l] = en[l] = 0.0;
    auto psi = [&](int l, int j, int i) -> float {
        if (j <= 0 || i <= 0 || j >= Ny - 1 || i >= Nx - 1) {
            if (!M.barotropic || j < 0 || i < 0 || j >= Ny || i >= Nx) return 0.f;
        }
        float p = 0.f;
        for (int m = 0; m < nl; ++m) p = fmaf(M.Cm2l[l * kMaxLayers + m], psi_hat[xrow_idx(M, m, j, i)], p);
        return p;
    };
    // u at V point (j, i) for interior j, i; zero elsewhere
    auto uV = [&](int l, int j, int i) -> float {
        if (j <= 0 || i <= 0 || j >= Ny - 1 || i >= Nx - 1) return 0.f;
        return -(psi(l, j + 1, i) - psi(l, j, i)) / M.dy;
    };
    auto vU = [&](int l, int j, int i) -> float {
        if (j <= 0 || i <= 0 || j >= Ny - 1 || i >= Nx - 1) return 0.f;
        return (psi(l, j, i + 1) - psi(l, j, i)) / M.dx;
    };
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j <= 0 || i <= 0 || j >= Ny - 1 || i >= Nx - 1) continue;
        for (int l = 0; l < nl; ++l) {
            const float uT = 0.5f * (uV(l, j, i) + uV(l, j - 1, i));
            const float vT = 0.5f * (vU(l, j, i) + vU(l, j, i - 1));
            ke[l] += (double)uT * uT + (double)vT * vT;
            const float qv = q[caller_idx(M, l, j, i)];
            en[l] += (double)qv * qv;
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int l = 0; l < nl; ++l) {
        double a = ke[l], b = en[l];
        for (int o = 16; o > 0; o >>= 1) {
            a += __shfl_down_sync(0xffffffffu, a, o);
            b += __shfl_down_sync(0xffffffffu, b, o);
        }
        if (lane == 0) {
            red[l][w] = a;
            red[kMaxLayers + l][w] = b;
        }
    }
    __syncthreads();
    if (threadIdx.x < nl) {
        const int l = threadIdx.x;
        double a = 0.0, b = 0.0;
        for (int k = 0; k < NTHREADS / 32; ++k) {
            a += red[l][k];
            b += red[kMaxLayers + l][k];
        }
        const double area = 0.5 * (double)M.dx * (double)M.dy;
        atomicAdd(&acc[2 * (M.off_layer + l)], a * area);
        atomicAdd(&acc[2 * (M.off_layer + l) + 1], b * area);
    }
}

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------
cudaError_t launch_prep(const MemberDev* members, const StencilTile* tiles, int ntiles,
                        const float* q, float* q_bc_inplace, int apply_bc, void* xa, int xa_fmt,
                        float* xq, int64_t xplane, cudaStream_t s) {
    k_prep<<<ntiles, NTHREADS, 0, s>>>(members, tiles, q, q_bc_inplace, apply_bc, xa, xa_fmt, xq,
                                       xplane);
    return cudaGetLastError();
}

void stencil_init() {
    cudaFuncSetAttribute(k_stencil, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)stencil_smem_bytes(kMaxLayers));
}

size_t stencil_smem_bytes(int max_nl) { return (size_t)3 * max_nl * SH * SW * sizeof(float); }

cudaError_t launch_stencil(const StencilArgs& a, int ntiles, int max_nl, int64_t xplane,
                           cudaStream_t s) {
    const size_t smem = stencil_smem_bytes(max_nl);
    k_stencil<<<ntiles, NTHREADS, smem, s>>>(a, xplane);
    return cudaGetLastError();
}

cudaError_t launch_mode_to_layer(const MemberDev* members, const StencilTile* tiles, int ntiles,
                                 const float* psi_hat, float* psi, cudaStream_t s) {
    k_mode_to_layer<<<ntiles, NTHREADS, 0, s>>>(members, tiles, psi_hat, psi);
    return cudaGetLastError();
}

cudaError_t launch_residual(const MemberDev* members, const StencilTile* tiles, int ntiles,
                            const float* qm, const float* psi_hat, void* out, int out_fmt,
                            int64_t xplane, cudaStream_t s) {
    k_residual<<<ntiles, NTHREADS, 0, s>>>(members, tiles, qm, psi_hat, out, out_fmt, xplane);
    return cudaGetLastError();
}

__global__ void k_diag_finish(const double* __restrict__ acc, int64_t n, float* ke, float* ens) {
    const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (l < n) {
        ke[l] = (float)acc[2 * l];
        ens[l] = (float)acc[2 * l + 1];
    }
}

cudaError_t launch_diag_finish(const double* acc, int64_t n_layers, float* ke, float* ens,
                               cudaStream_t s) {
    k_diag_finish<<<(unsigned)((n_layers + 127) / 128), 128, 0, s>>>(acc, n_layers, ke, ens);
    return cudaGetLastError();
}

cudaError_t launch_diag_acc(const MemberDev* members, const StencilTile* tiles, int ntiles,
                            const float* q, const float* psi_hat, double* acc, cudaStream_t s) {
    k_diag<<<ntiles, NTHREADS, 0, s>>>(members, tiles, q, psi_hat, acc);
    return cudaGetLastError();
}

}  // namespace qg
