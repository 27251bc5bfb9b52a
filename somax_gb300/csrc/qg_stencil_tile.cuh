// One tile of the fused RHS stencil, shared by the stand-alone stencil kernel
// (qg_stencil.cu) and the persistent step kernel (qg_persistent.cu).  A tile is TX x TY
// interior cells of one member, all layers, computed by 256 threads from TMA boxes of q and
// psi_hat with a two-cell halo (x from tx0 - 4 so the box starts on a 16-byte boundary).
// Two tile shapes: 32 x 8 (one cell per thread: short latency chains and many CTAs for small
// grids) and 64 x 16 (four cells per thread: less halo traffic for large grids).
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {
namespace st {

constexpr int NTHREADS = 256;

template <int TX_, int TY_>
struct Tile {
    static constexpr int TX = TX_;                   // interior tile width  (x)
    static constexpr int TY = TY_;                   // interior tile height (y)
    static constexpr int BX = TX + 8;                // box width: x from tx0 - 4 (16-byte aligned)
    static constexpr int BY = TY + 4;                // box height: two halo rows each side
    static constexpr int BOX = BX * BY;              // floats per layer in a box
    static constexpr int PER_THREAD = TX * TY / NTHREADS;
    static_assert(TX * TY % NTHREADS == 0, "tile cells must split evenly over the threads");
    static_assert(BX * 4 % 16 == 0, "TMA box rows must be whole 16-byte units");
};
using TileS = Tile<32, 8>;
using TileL = Tile<64, 16>;

struct StencilMaps {
    CUtensorMap q[3];  // stage planes S0, S1, S2
    CUtensorMap psi;   // psi_hat plane
};
static_assert(sizeof(StencilMaps) == kStencilMapsBytes, "StencilMaps size");

// Shared memory of one tile: q and psi boxes (TMA destinations) and lap(q) (computed).
template <class T>
__host__ __device__ constexpr size_t tile_box_bytes(int nl) {
    return (size_t)2 * nl * T::BOX * sizeof(float);
}
template <class T>
__host__ __device__ constexpr size_t tile_lap_bytes(int nl) {
    return (size_t)nl * T::BOX * sizeof(float);
}

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

// Issue the two TMA box copies of tile (ty, tx) of a member: q from stage plane `q_sel` and
// psi_hat, all layers, completing on `bar`.
template <class T>
__device__ __forceinline__ void tile_issue(const StencilMaps* maps, int q_sel, int nl, int ty, int tx, float* sq,
                                           float* sp, uint64_t* bar) {
    mbar_expect_tx(bar, (uint32_t)tile_box_bytes<T>(nl));
    tma_load_3d(sq, &maps->q[q_sel], bar, tx * T::TX - 4, ty * T::TY - 2, 0);
    tma_load_3d(sp, &maps->psi, bar, tx * T::TX - 4, ty * T::TY - 2, 0);
}

// After the TMA boxes landed: zero the q ring (BC on read), mix psi_hat to layer psi in
// place zeroing the baroclinic psi ring (baroclinic.py:155-158), and lap(q) of the cells one
// ring beyond the tile (zero on the ghost ring: the interior-only Laplacian).  NL = layers.
template <class T, int NL>
__device__ __forceinline__ void stencil_fix_box(const MemberDev& M, float* sq, float* sp, float* sl, int ty, int tx,
                                                int apply_bc, bool need_lap) {
    constexpr int BX = T::BX, BOX = T::BOX;
    const int Ny = M.Ny, Nx = M.Nx;
    const int j0 = ty * T::TY - 2, i0 = tx * T::TX - 4;
    const bool edge = (j0 <= 0) || (i0 <= 0) || (j0 + T::BY >= Ny) || (i0 + BX >= Nx);
    const uint8_t* mask = M.mask;  // in a register: the loops below store to shared memory
    float C[NL][NL];
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
        for (int m = 0; m < NL; ++m) C[l][m] = M.Cm2l[l * kMaxLayers + m];
    for (int c = threadIdx.x; c < BOX; c += NTHREADS) {
        const int j = j0 + c / BX, i = i0 + c % BX;
        const bool ring = edge && j >= 0 && j < Ny && i >= 0 && i < Nx && on_ring(j, i, Ny, Nx);
        const bool land = is_land(mask, Ny, Nx, j, i);  // q and psi are zero on land
        if ((apply_bc && ring) || land)
#pragma unroll
            for (int l = 0; l < NL; ++l) sq[l * BOX + c] = 0.f;
        float ph[NL];
#pragma unroll
        for (int m = 0; m < NL; ++m) ph[m] = sp[m * BOX + c];
        const bool zero = (ring && !M.barotropic) || land;
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            float p = 0.f;
#pragma unroll
            for (int m = 0; m < NL; ++m) p = fmaf(C[l][m], ph[m], p);
            sp[l * BOX + c] = zero ? 0.f : p;
        }
    }
    if (!need_lap) return;
    __syncthreads();  // lap(q) reads the BC'd neighbours
    const float idx2 = M.inv_dx2, idy2 = M.inv_dy2;
    constexpr int LW = T::TX + 2, LH = T::TY + 2;  // cells one beyond the tile
    for (int c = threadIdx.x; c < LW * LH; c += NTHREADS) {
        const int sy = 1 + c / LW, sx = 3 + c % LW;  // box coordinates
        const int j = j0 + sy, i = i0 + sx;
        const bool interior = j > 0 && i > 0 && j < Ny - 1 && i < Nx - 1 && !is_land(mask, Ny, Nx, j, i);
        const int b = sy * BX + sx;
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            const float* Q = sq + l * BOX + b;
            sl[l * BOX + b] = interior ? (Q[1] - 2.f * Q[0] + Q[-1]) * idx2 + (Q[BX] - 2.f * Q[0] + Q[-BX]) * idy2
                                       : 0.f;
        }
    }
}

// Compute the tile's cells from the fixed boxes: rhs mode writes dq, step mode writes the
// stage update, the next stage's modal operand and its FP32 copy.  y0 of every cell of the
// thread is loaded before any arithmetic.  Returns true if a non-finite value was produced.
template <class T, int NL>
__device__ __forceinline__ bool stencil_compute(const StencilArgs& a, const MemberDev& M, const StencilTile& t,
                                                const float* sq, const float* sp, const float* sl) {
    constexpr int BX = T::BX, BOX = T::BOX, R = T::PER_THREAD;
    // member constants in registers: the stores below go through generic pointers, after which
    // the compiler would otherwise reload every field of M from shared memory
    const int Ny = M.Ny, Nx = M.Nx, Px = M.Px;
    const uint8_t* mask = M.mask;
    const float i12 = M.inv_12dxdy, b12 = M.beta_12dx, invH0 = M.invH0;
    const int64_t off_x = M.off_x, off_c = M.off_state;
    const int64_t lsx = (int64_t)Ny * Px, lsc = (int64_t)Ny * Nx;
    const float* P = a.params + (int64_t)t.member * QG_NPARAMS;
    const float nu = P[QG_P_NU], kappa = P[QG_P_KAPPA], tau0 = P[QG_P_TAU0], nu4 = P[QG_P_NU4];
    const float idx2 = M.inv_dx2, idy2 = M.inv_dy2;
    const int lx = threadIdx.x % T::TX;
    const int ly0 = (threadIdx.x / T::TX) * R;
    const int i = t.tx * T::TX + lx;
    const bool step = a.dq == nullptr;
    float y0r[R][NL];
    float Fj[R];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int j = t.ty * T::TY + ly0 + r;
        const bool in = j < Ny && i < Nx;
        Fj[r] = in ? M.F[j] : 0.f;
#pragma unroll
        for (int l = 0; l < NL; ++l) y0r[r][l] = (step && in) ? a.y0[off_x + l * lsx + (int64_t)j * Px + i] : 0.f;
    }
    bool bad = false;
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int ly = ly0 + r;
        const int j = t.ty * T::TY + ly;
        if (j >= Ny || i >= Nx) continue;
        const bool ring = on_ring(j, i, Ny, Nx);
        const bool land = is_land(mask, Ny, Nx, j, i);  // no dynamics on land
        const int s0 = (ly + 2) * BX + (lx + 4);  // box index of the cell
        const float wind = tau0 * Fj[r] * invH0;
        const int64_t xo = off_x + (int64_t)j * Px + i, co = off_c + (int64_t)j * Nx + i;
        float d[NL];
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            if (ring || land) {
                d[l] = (ring && l == 0) ? wind : 0.f;
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
            const float Jq = (jpp + jpx + jxp) * i12;
            const float Jb = (4.f * (fE - fW) + (fNE - fNW) + (fSE - fSW)) * b12;
            float v = -(Jq + Jb);
            if (l == 0) v += wind;
            if (l == NL - 1) {
                const float lp = (fE - 2.f * S[0] + fW) * idx2 + (fN - 2.f * S[0] + fS) * idy2;
                v += -kappa * lp;
            }
            const float lq = (gE - 2.f * Q[0] + gW) * idx2 + (gN - 2.f * Q[0] + gS) * idy2;
            v += nu * lq;
            if (nu4 != 0.f) {
                // lap(lap q) from lap(q) in shared memory (zero on the ghost ring)
                const float* L = sl + l * BOX + s0;
                const float bl = (L[1] - 2.f * L[0] + L[-1]) * idx2 + (L[BX] - 2.f * L[0] + L[-BX]) * idy2;
                v -= nu4 * bl;
            }
            d[l] = v;
        }
#pragma unroll
        for (int l = 0; l < NL; ++l) bad |= !isfinite(d[l]);

        if (!step) {
#pragma unroll
            for (int l = 0; l < NL; ++l) a.dq[co + l * lsc] = d[l];
            continue;
        }
        float yn[NL];
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            if (ring) {
                // The ring tendency is state independent (wind only), so every consistent
                // RK scheme ends at y0 + dt * dq there; stage inputs carry a zero ring (BC).
                yn[l] = a.final_stage ? y0r[r][l] + a.dt * d[l] : 0.f;
            } else {
                yn[l] = a.a * y0r[r][l] + a.b * (sq[l * BOX + s0] + a.dt * d[l]);
            }
            bad |= !isfinite(yn[l]);
            a.y_next[xo + l * lsx] = yn[l];
        }
        if (a.xa) {
#pragma unroll
            for (int m = 0; m < NL; ++m) {
                float s = 0.f;
                if (!ring && !land)
#pragma unroll
                    for (int l = 0; l < NL; ++l) s = fmaf(M.Cl2m[m * kMaxLayers + l], yn[l], s);
                store_plane(a.xa, a.xa_fmt, a.xplane, xo + m * lsx, s);
                if (a.xq) a.xq[xo + m * lsx] = s;
            }
        }
    }
    return bad;
}

// Fix the boxes of one tile and compute it; dispatches on the member's layer count.
template <class T>
__device__ __forceinline__ bool stencil_tile(const StencilArgs& a, const MemberDev& M, const StencilTile& t,
                                             float* sq, float* sp, float* sl, int apply_bc, bool need_lap) {
#define QG_NL_CASE(N)                                                \
    case N:                                                          \
        stencil_fix_box<T, N>(M, sq, sp, sl, t.ty, t.tx, apply_bc, need_lap); \
        __syncthreads();                                             \
        return stencil_compute<T, N>(a, M, t, sq, sp, sl);
    switch (M.nl) {
        QG_NL_CASE(1)
        QG_NL_CASE(2)
        QG_NL_CASE(3)
        QG_NL_CASE(4)
        QG_NL_CASE(5)
        QG_NL_CASE(6)
        QG_NL_CASE(7)
        QG_NL_CASE(8)
        default:
            return true;
    }
#undef QG_NL_CASE
}

}  // namespace st
}  // namespace qg
