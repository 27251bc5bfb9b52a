// Memory-bound kernels of the QG time step: the fused RHS stencil (with the RK stage update
// and the next stage's layer->mode prologue fused in), the pack / unpack of the state into
// the padded internal planes, the mode->layer epilogue, the Helmholtz residual and the
// diagnostics.
//
// Every kernel walks a list of 2-D tiles (StencilTile) that may belong to different members
// of an ensemble; a block owns one tile and all layers of it.  Kernels start with the
// programmatic-dependent-launch handshake: constants are read before griddepcontrol.wait,
// anything a predecessor kernel writes only after it.
#include <cuda_bf16.h>

#include <cstring>

#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {

namespace {

constexpr int TX = kStencilTX;      // interior tile width  (x)
constexpr int TY = kStencilTY;      // interior tile height (y)
constexpr int BX = TX + 8;          // TMA box width: x from tx0 - 4 (16-byte aligned start)
constexpr int BY = TY + 4;          // box height: two halo rows each side (biharmonic)
constexpr int BOX = BX * BY;        // floats per layer in a box
constexpr int NTHREADS = 256;
constexpr int ROWS_PER_THREAD = TX * TY / NTHREADS;  // 4

struct StencilMaps {
    CUtensorMap q[3];  // stage planes S0, S1, S2
    CUtensorMap psi;   // psi_hat plane
};
static_assert(sizeof(StencilMaps) == kStencilMapsBytes, "StencilMaps size");

// Copy a member's constants into shared memory (one 4-byte word per thread per pass).
__device__ __forceinline__ void load_member(MemberDev* dst, const MemberDev* src) {
    const int* s = reinterpret_cast<const int*>(src);
    int* d = reinterpret_cast<int*>(dst);
    for (int w = threadIdx.x; w < (int)(sizeof(MemberDev) / 4); w += blockDim.x) d[w] = s[w];
}

__device__ __forceinline__ bool on_ring(int j, int i, int Ny, int Nx) {
    return j == 0 || i == 0 || j == Ny - 1 || i == Nx - 1;
}

// Index of (l, j, i) in a packed caller field / in an internal x-row plane.
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
// Pack: copy q (caller packing) into an internal plane (optionally zeroing its ring) and
// write the layer->mode operand Cl2m q (BC applied when bc_operand) for the DST GEMMs.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_prep(PrepArgs a) {
    __shared__ MemberDev M;
    const StencilTile t = a.tiles[blockIdx.x];
    load_member(&M, a.members + t.member);
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();
    const int nl = M.nl;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        const bool ring = on_ring(j, i, M.Ny, M.Nx);
        float v[kMaxLayers];
        for (int l = 0; l < nl; ++l) {
            const float x = a.q[caller_idx(M, l, j, i)];
            if (a.copy) a.copy[xrow_idx(M, l, j, i)] = (a.zero_ring_copy && ring) ? 0.f : x;
            v[l] = (a.bc_operand && ring) ? 0.f : x;
        }
        if (!a.xa) continue;
        for (int m = 0; m < nl; ++m) {
            float s = 0.f;
            for (int l = 0; l < nl; ++l) s = fmaf(M.Cl2m[m * kMaxLayers + l], v[l], s);
            store_plane(a.xa, a.xa_fmt, a.xplane, xrow_idx(M, m, j, i), s);
            if (a.xq) a.xq[xrow_idx(M, m, j, i)] = s;
        }
    }
}

// Unpack: internal plane -> caller packing (every cell, ring included).
__global__ void __launch_bounds__(NTHREADS) k_unpack(const MemberDev* __restrict__ members,
                                                     const StencilTile* __restrict__ tiles,
                                                     const float* __restrict__ src, float* __restrict__ q) {
    __shared__ MemberDev M;
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        for (int l = 0; l < M.nl; ++l) q[caller_idx(M, l, j, i)] = src[xrow_idx(M, l, j, i)];
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
//
// The halo tile of q and psi_hat, all layers, arrives by two 3-D TMA copies (zero fill
// outside the array).  Step mode fuses the Shu-Osher stage update
// y_next = a y0 + b (y_s + dt dq) and the next stage's layer->mode prologue.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_stencil(StencilArgs a) {
    extern __shared__ uint8_t smem_raw[];
    float* smem = reinterpret_cast<float*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
    __shared__ MemberDev M;
    __shared__ __align__(8) uint64_t bar;
    __shared__ int abort_flag;
    const StencilTile t = a.tiles[blockIdx.x];
    const StencilMaps* maps = static_cast<const StencilMaps*>(a.maps) + t.member;
    load_member(&M, a.members + t.member);
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_init_fence();
        abort_flag = 0;
        tma_prefetch_desc(&maps->q[a.q_sel]);
        tma_prefetch_desc(&maps->psi);
    }
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();

    const int nl = M.nl, Ny = M.Ny, Nx = M.Nx;
    float* sq = smem;              // [nl][BY][BX] q, then BC applied
    float* sp = smem + nl * BOX;   // [nl][BY][BX] psi_hat, mixed in place to psi
    const int j0 = t.ty * TY - 2, i0 = t.tx * TX - 4;
    if (threadIdx.x == 0) {
        mbar_expect_tx(&bar, (uint32_t)(2 * nl * BOX * sizeof(float)));
        tma_load_3d(sq, &maps->q[a.q_sel], &bar, i0, j0, 0);
        tma_load_3d(sp, &maps->psi, &bar, i0, j0, 0);
    }
    const bool have = mbar_wait(&bar, 0, &abort_flag);
    const float* P = a.params + (int64_t)t.member * QG_NPARAMS;
    const float nu = P[QG_P_NU], kappa = P[QG_P_KAPPA], tau0 = P[QG_P_TAU0], nu4 = P[QG_P_NU4];

    // BC on the q ring; psi = Cm2l psi_hat with the baroclinic ring zeroed
    const bool edge = (j0 <= 0) || (i0 <= 0) || (j0 + BY >= Ny) || (i0 + BX >= Nx);
    for (int c = threadIdx.x; c < BOX; c += blockDim.x) {
        const int j = j0 + c / BX, i = i0 + c % BX;
        const bool ring = edge && j >= 0 && j < Ny && i >= 0 && i < Nx && on_ring(j, i, Ny, Nx);
        if (a.apply_bc && ring)
            for (int l = 0; l < nl; ++l) sq[l * BOX + c] = 0.f;
        if (nl > 1) {
            float ph[kMaxLayers];
            for (int m = 0; m < nl; ++m) ph[m] = sp[m * BOX + c];
            for (int l = 0; l < nl; ++l) {
                float p = 0.f;
                for (int m = 0; m < nl; ++m) p = fmaf(M.Cm2l[l * kMaxLayers + m], ph[m], p);
                sp[l * BOX + c] = p;
            }
        } else if (M.Cm2l[0] != 1.f) {
            sp[c] *= M.Cm2l[0];
        }
        if (ring && !M.barotropic)
            for (int l = 0; l < nl; ++l) sp[l * BOX + c] = 0.f;
    }
    __syncthreads();

    const float idx2 = M.inv_dx2, idy2 = M.inv_dy2;
    const int lx = threadIdx.x % TX;
    const int ly0 = (threadIdx.x / TX) * ROWS_PER_THREAD;
    const int i = t.tx * TX + lx;
    bool bad = !have;
#pragma unroll 1
    for (int r = 0; r < ROWS_PER_THREAD; ++r) {
        const int ly = ly0 + r;
        const int j = t.ty * TY + ly;
        if (j >= Ny || i >= Nx) continue;
        const bool ring = on_ring(j, i, Ny, Nx);
        const int s0 = (ly + 2) * BX + (lx + 4);  // box index of the cell
        const float wind = tau0 * M.F[j] * M.invH0;
        float d[kMaxLayers];
        for (int l = 0; l < nl; ++l) {
            if (ring) {
                d[l] = (l == 0) ? wind : 0.f;
                continue;
            }
            const float* Q = sq + l * BOX + s0;
            const float* S = sp + l * BOX + s0;
            const float fE = S[1], fW = S[-1], fN = S[BX], fS = S[-BX];
            const float fNE = S[BX + 1], fNW = S[BX - 1], fSE = S[-BX + 1], fSW = S[-BX - 1];
            const float gE = Q[1], gW = Q[-1], gN = Q[BX], gS = Q[-BX];
            const float gNE = Q[BX + 1], gNW = Q[BX - 1], gSE = Q[-BX + 1], gSW = Q[-BX - 1];
            const float jpp = (fE - fW) * (gN - gS) - (fN - fS) * (gE - gW);
            const float jpx = fE * (gNE - gSE) - fW * (gNW - gSW) - fN * (gNE - gNW) + fS * (gSE - gSW);
            const float jxp = gN * (fNE - fNW) - gS * (fSE - fSW) - gE * (fNE - fSE) + gW * (fNW - fSW);
            const float Jq = (jpp + jpx + jxp) * M.inv_12dxdy;
            const float Jb = (4.f * (fE - fW) + (fNE - fNW) + (fSE - fSW)) * M.beta_12dx;
            float v = -(Jq + Jb);
            if (l == 0) v += wind;
            if (l == nl - 1) {
                const float lp = (fE - 2.f * S[0] + fW) * idx2 + (fN - 2.f * S[0] + fS) * idy2;
                v += -kappa * lp;
            }
            const float lq = (gE - 2.f * Q[0] + gW) * idx2 + (gN - 2.f * Q[0] + gS) * idy2;
            v += nu * lq;
            if (nu4 != 0.f) {
                // lap(lap q) with lap(q) = 0 on the ring (interior-only Laplacian)
                auto lap_at = [&](int dj, int di) -> float {
                    const int jj = j + dj, ii = i + di;
                    if (jj <= 0 || ii <= 0 || jj >= Ny - 1 || ii >= Nx - 1) return 0.f;
                    const float* c = Q + dj * BX + di;
                    return (c[1] - 2.f * c[0] + c[-1]) * idx2 + (c[BX] - 2.f * c[0] + c[-BX]) * idy2;
                };
                const float l0 = lap_at(0, 0);
                const float bl = (lap_at(0, 1) - 2.f * l0 + lap_at(0, -1)) * idx2 +
                                 (lap_at(1, 0) - 2.f * l0 + lap_at(-1, 0)) * idy2;
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
            const int64_t o = xrow_idx(M, l, j, i);
            const float y0 = a.y0[o];
            if (ring) {
                // The ring tendency is state independent (wind only), so every consistent
                // RK scheme ends at y0 + dt * dq there; stage inputs carry a zero ring (BC).
                yn[l] = a.final_stage ? y0 + a.dt * d[l] : 0.f;
            } else {
                yn[l] = a.a * y0 + a.b * (sq[l * BOX + s0] + a.dt * d[l]);
            }
            bad |= !isfinite(yn[l]);
            a.y_next[o] = yn[l];
        }
        if (a.xa) {
            for (int m = 0; m < nl; ++m) {
                float s = 0.f;
                if (!ring)
                    for (int l = 0; l < nl; ++l) s = fmaf(M.Cl2m[m * kMaxLayers + l], yn[l], s);
                store_plane(a.xa, a.xa_fmt, a.xplane, xrow_idx(M, m, j, i), s);
                if (a.xq) a.xq[xrow_idx(M, m, j, i)] = s;
            }
        }
    }
    if (bad && a.flags) atomicOr(a.flags, have ? 1 : 2);
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
    pdl_wait();
    pdl_launch_dependents();
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
    pdl_wait();
    pdl_launch_dependents();
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
    pdl_wait();
    pdl_launch_dependents();
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
        double x = ke[l], y = en[l];
        for (int o = 16; o > 0; o >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, o);
            y += __shfl_down_sync(0xffffffffu, y, o);
        }
        if (lane == 0) {
            red[l][w] = x;
            red[kMaxLayers + l][w] = y;
        }
    }
    __syncthreads();
    if (threadIdx.x < nl) {
        const int l = threadIdx.x;
        double x = 0.0, y = 0.0;
        for (int k = 0; k < NTHREADS / 32; ++k) {
            x += red[l][k];
            y += red[kMaxLayers + l][k];
        }
        const double area = 0.5 * (double)M.dx * (double)M.dy;
        atomicAdd(&acc[2 * (M.off_layer + l)], x * area);
        atomicAdd(&acc[2 * (M.off_layer + l) + 1], y * area);
    }
}

__global__ void k_diag_finish(const double* __restrict__ acc, int64_t n, float* ke, float* ens) {
    pdl_wait();
    pdl_launch_dependents();
    const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (l < n) {
        ke[l] = (float)acc[2 * l];
        ens[l] = (float)acc[2 * l + 1];
    }
}

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------
size_t stencil_smem_bytes(int max_nl) { return (size_t)2 * max_nl * BOX * sizeof(float) + 128; }

// 3-D boxes (BX, BY, nl) over a member's x-row planes: dims (Nx, Ny, nl), row pitch Px.
cudaError_t stencil_encode_maps(const MemberDev& M, const float* const planes[4], void* out) {
    StencilMaps sm;
    memset(&sm, 0, sizeof(sm));
    const uint64_t dims[3] = {(uint64_t)M.Nx, (uint64_t)M.Ny, (uint64_t)M.nl};
    const uint64_t strides[2] = {(uint64_t)M.Px * 4, (uint64_t)M.Px * M.Ny * 4};
    const uint32_t box[3] = {(uint32_t)BX, (uint32_t)BY, (uint32_t)M.nl};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 4 && !e; ++k) {
        CUtensorMap* m = k < 3 ? &sm.q[k] : &sm.psi;
        e = tmap_encode(m, 0, 3, planes[k] + M.off_x, dims, strides, box, 0);
    }
    if (!e) memcpy(out, &sm, sizeof(sm));
    return e;
}

void stencil_init() {
    cudaFuncSetAttribute(k_stencil, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         (int)stencil_smem_bytes(kMaxLayers));
}

cudaError_t launch_prep(const PrepArgs& a, int ntiles, cudaStream_t s, bool pdl) {
    return launch_k(k_prep, ntiles, NTHREADS, 0, s, pdl, a);
}

cudaError_t launch_unpack(const MemberDev* members, const StencilTile* tiles, int ntiles, const float* src,
                          float* q, cudaStream_t s, bool pdl) {
    return launch_k(k_unpack, ntiles, NTHREADS, 0, s, pdl, members, tiles, src, q);
}

cudaError_t launch_stencil(const StencilArgs& a, int ntiles, int max_nl, cudaStream_t s, bool pdl) {
    return launch_k(k_stencil, ntiles, NTHREADS, stencil_smem_bytes(max_nl), s, pdl, a);
}

cudaError_t launch_mode_to_layer(const MemberDev* members, const StencilTile* tiles, int ntiles,
                                 const float* psi_hat, float* psi, cudaStream_t s, bool pdl) {
    return launch_k(k_mode_to_layer, ntiles, NTHREADS, 0, s, pdl, members, tiles, psi_hat, psi);
}

cudaError_t launch_residual(const MemberDev* members, const StencilTile* tiles, int ntiles,
                            const float* qm, const float* psi_hat, void* out, int out_fmt,
                            int64_t xplane, cudaStream_t s, bool pdl) {
    return launch_k(k_residual, ntiles, NTHREADS, 0, s, pdl, members, tiles, qm, psi_hat, out, out_fmt, xplane);
}

cudaError_t launch_diag_acc(const MemberDev* members, const StencilTile* tiles, int ntiles,
                            const float* q, const float* psi_hat, double* acc, cudaStream_t s) {
    return launch_k(k_diag, ntiles, NTHREADS, 0, s, false, members, tiles, q, psi_hat, acc);
}

cudaError_t launch_diag_finish(const double* acc, int64_t n_layers, float* ke, float* ens,
                               cudaStream_t s) {
    return launch_k(k_diag_finish, (int)((n_layers + 127) / 128), 128, 0, s, false, acc, n_layers, ke, ens);
}

}  // namespace qg
