// One tile of the fused RHS stencil, shared by the stand-alone stencil kernel
// (qg_stencil.cu) and the persistent step kernel (qg_persistent.cu).  A tile is TX x TY
// interior cells of one member, all layers, computed by 256 threads from TMA boxes of q and
// psi_hat with a two-cell halo (x from tx0 - 4 so the box starts on a 16-byte boundary).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {
namespace st {

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


// After the TMA boxes landed: zero the q ring (BC on read) and mix psi_hat to layer psi in
// place, zeroing the baroclinic psi ring (baroclinic.py:155-158).
__device__ __forceinline__ void stencil_fix_box(const MemberDev& M, float* sq, float* sp, int j0, int i0,
                                                int apply_bc) {
    const int nl = M.nl, Ny = M.Ny, Nx = M.Nx;
    // BC on the q ring; psi = Cm2l psi_hat with the baroclinic ring zeroed
    const bool edge = (j0 <= 0) || (i0 <= 0) || (j0 + BY >= Ny) || (i0 + BX >= Nx);
    for (int c = threadIdx.x; c < BOX; c += blockDim.x) {
        const int j = j0 + c / BX, i = i0 + c % BX;
        const bool ring = edge && j >= 0 && j < Ny && i >= 0 && i < Nx && on_ring(j, i, Ny, Nx);
        if (apply_bc && ring)
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
}

// Compute the tile's cells from the fixed boxes: rhs mode writes dq, step mode writes the
// stage update, the next stage's modal operand and its FP32 copy.  Returns true if a
// non-finite value was produced.
__device__ __forceinline__ bool stencil_compute(const StencilArgs& a, const MemberDev& M, const StencilTile& t,
                                                const float* sq, const float* sp) {
    const int nl = M.nl, Ny = M.Ny, Nx = M.Nx;
    const float* P = a.params + (int64_t)t.member * QG_NPARAMS;
    const float nu = P[QG_P_NU], kappa = P[QG_P_KAPPA], tau0 = P[QG_P_TAU0], nu4 = P[QG_P_NU4];
    const float idx2 = M.inv_dx2, idy2 = M.inv_dy2;
    const int lx = threadIdx.x % TX;
    const int ly0 = (threadIdx.x / TX) * ROWS_PER_THREAD;
    const int i = t.tx * TX + lx;
    bool bad = false;
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
    return bad;
}

}  // namespace st
}  // namespace qg
