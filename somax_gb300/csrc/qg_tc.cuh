// tcgen05 building blocks of the DST-I GEMMs, shared by the one-tile-per-CTA kernels
// (qg_gemm_tc.cu) and the persistent step kernel (qg_persistent.cu).
//
// C = A * S with A rows (layer, r) K-major and S symmetric (so its rows are the K-major B
// operand).  Operands are 128-byte rows in 128-byte-swizzled shared memory (the layout TMA
// writes with SWIZZLE_128B); the FP32 accumulator is a 128-lane x BN-column TMEM block.
#pragma once

#include <cuda.h>
#include <cuda_bf16.h>

#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {

constexpr int TC_BM = 128;
// Largest output tile width (N): 144 = 9 x 16 so that the N = n + 2 sizes of the DST (66,
// 130, 258, 514) need one, one, two and four tiles; a plan may cut narrower tiles (more
// CTAs for small members), and the last tile of a member runs its MMAs at the width it needs
// (a multiple of 16), so little of the tensor work is padding.  The S operand's TMA box is
// always TC_BN rows.
constexpr int TC_BN = 144;
constexpr int TC_TMEM_BUF = 256;   // TMEM column stride of the two accumulators
constexpr int TC_TMEM_COLS = 512;  // allocation (power of two >= 2 buffers)
// Width of output tile nt of a pass with Nn columns cut into tiles of bn (<= TC_BN) columns.
__host__ __device__ constexpr int tc_tile_width(int Nn, int nt, int bn) {
    return (Nn - nt * bn >= bn) ? bn : ((Nn - nt * bn + 15) / 16) * 16;
}

struct TcMaps {
    CUtensorMap a[2];  // A hi (or f32), A lo
    CUtensorMap b[2];  // S hi (or f32), S lo
};
static_assert(sizeof(TcMaps) == kTcMapsBytes, "TcMaps size");

template <int PREC>
struct TcCfg;
template <>
struct TcCfg<QG_DST_TF32> {
    static constexpr int BK = 32;  // 32 fp32 = 128-byte rows
    static constexpr int STAGES = 4;
    static constexpr int ESIZE = 4;
    static constexpr int NA = 1, NB = 1;  // operand planes
    static constexpr int UMMA_K = 8;      // 32 bytes per MMA along K
    static constexpr uint32_t FMT = 2;    // tf32
};
template <>
struct TcCfg<QG_DST_BF16X3> {
    static constexpr int BK = 64;  // 64 bf16 = 128-byte rows
    static constexpr int STAGES = 3;
    static constexpr int ESIZE = 2;
    static constexpr int NA = 2, NB = 2;  // hi, lo
    static constexpr int UMMA_K = 16;
    static constexpr uint32_t FMT = 1;    // bf16
};

template <int PREC>
__host__ __device__ constexpr int tc_tile_a_bytes() { return TC_BM * TcCfg<PREC>::BK * TcCfg<PREC>::ESIZE; }
template <int PREC>
__host__ __device__ constexpr int tc_tile_b_bytes() { return TC_BN * TcCfg<PREC>::BK * TcCfg<PREC>::ESIZE; }
template <int PREC>
__host__ __device__ constexpr int tc_stage_bytes() {
    return TcCfg<PREC>::NA * tc_tile_a_bytes<PREC>() + TcCfg<PREC>::NB * tc_tile_b_bytes<PREC>();
}

// Instruction descriptor: D f32, A/B format FMT, both K-major, N = n (a multiple of 16 up to
// TC_BN), M = TC_BM.
template <int PREC>
__device__ __forceinline__ uint32_t tc_idesc(int n) {
    return (1u << 4) | (TcCfg<PREC>::FMT << 7) | (TcCfg<PREC>::FMT << 10) | ((uint32_t)(n >> 3) << 17) |
           ((uint32_t)(TC_BM >> 4) << 24);
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row groups 1024
// bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
    d |= (uint64_t)1 << 46;            // version
    d |= (uint64_t)2 << 61;            // SWIZZLE_128B
    return d;
}

template <uint32_t FMT>
__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
    if constexpr (FMT == 2) {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(da), "l"(db), "r"(idesc), "r"(acc));
    } else {
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
            "l"(da), "l"(db), "r"(idesc), "r"(acc));
    }
}
__device__ __forceinline__ void tc_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(slot)), "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}
__device__ __forceinline__ void tc_dealloc(uint32_t tmem, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(ncols));
}
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(su32(b)) : "memory");
}

#define QG_LD32(r, taddr)                                                                                   \
    asm volatile(                                                                                           \
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"    \
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"                          \
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),  \
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),         \
          "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]),       \
          "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]),       \
          "=r"(r[29]), "=r"(r[30]), "=r"(r[31])                                                            \
        : "r"(taddr))

// Geometry of a pass for one member: A rows (l, r) of Mb rows a layer, K contracted, output
// C^T[l][n][r] with row pitch ldo in the other orientation's planes.
struct TcGeom {
    int Mb, K, Nn, Mtot, ldo;
    int64_t cbase, cplane;
};
template <int PASS>
__device__ __forceinline__ TcGeom tc_geom(const MemberDev& M, int64_t xplane, int64_t yplane) {
    constexpr bool xin = pass_xin(PASS);
    TcGeom g;
    g.Mb = xin ? M.Ny : M.Nx;
    g.K = xin ? M.Nx : M.Ny;
    g.Nn = g.K;
    g.Mtot = M.nl * g.Mb;
    g.ldo = xin ? M.Py : M.Px;
    g.cbase = xin ? M.off_y : M.off_x;
    g.cplane = xin ? yplane : xplane;
    return g;
}

// What the drain of one output tile reads besides its accumulator: the pass geometry, the
// tile's first row and column and width, and (G2) the member's eigenvalue tables.
struct TcTile {
    TcGeom g;
    const float* ex;   // DST-I eigenvalues along the output rows' axis (G2)
    const float* ey;   // along the output columns' axis (G2)
    const float* lam;  // modal Helmholtz constants per layer (G2)
    int member, m0, n0, width;
};
template <int PASS>
__device__ __forceinline__ TcTile tc_tile(const MemberDev* members, const GemmTile& tl, int64_t xplane, int64_t yplane,
                                          int tile_n) {
    TcTile t;
    t.member = tl.member;
    if (tl.member < 0) return t;  // a padding entry of the balanced schedule: nothing is read
    const MemberDev& M = members[tl.member];
    t.g = tc_geom<PASS>(M, xplane, yplane);
    t.ex = M.ex;
    t.ey = M.ey;
    t.lam = M.lam;
    t.m0 = tl.mt * TC_BM;
    t.n0 = tl.nt * tile_n;
    t.width = tc_tile_width(t.g.Nn, tl.nt, tile_n);
    return t;
}

// G2's divisor row term ex[r] - lam[l] of the accumulator row that `lane` of lane quarter
// `quarter` holds (0 for the other passes and for rows past the member's last).
template <int PASS>
__device__ __forceinline__ float tc_rowterm(const TcTile& T, int quarter, int lane) {
    if constexpr (PASS != G2_FWD_Y) return 0.f;
    const int m = T.m0 + quarter * 32 + lane;
    if (m >= T.g.Mtot) return 0.f;
    const int l = m / T.g.Mb;
    return T.ex[m - l * T.g.Mb] - T.lam[l];
}

// Issue the MMAs of one k-block (operands at shared addresses sa / sb) into tmem_d: `ksteps`
// UMMA_K-wide steps (the last k-block of a member stops at its K; the zero fill beyond it
// contributes nothing) at output width n.
template <int PREC>
__device__ __forceinline__ void tc_mma_kblock(uint32_t tmem_d, uint32_t sa, uint32_t sb, bool first, int ksteps,
                                              int n) {
    using C = TcCfg<PREC>;
    const uint32_t idesc = tc_idesc<PREC>(n);
#pragma unroll
    for (int k = 0; k < C::BK / C::UMMA_K; ++k) {
        if (k >= ksteps) break;
        const uint32_t koff = k * C::UMMA_K * C::ESIZE;  // 32 bytes per step
        const uint64_t a0 = tc_sdesc(sa + koff), b0 = tc_sdesc(sb + koff);
        tc_mma<C::FMT>(tmem_d, a0, b0, idesc, (!first || k > 0) ? 1u : 0u);
        if constexpr (C::NA == 2) {
            const uint64_t a1 = tc_sdesc(sa + tc_tile_a_bytes<PREC>() + koff);
            const uint64_t b1 = tc_sdesc(sb + tc_tile_b_bytes<PREC>() + koff);
            tc_mma<C::FMT>(tmem_d, a0, b1, idesc, 1u);  // Ahi * Slo
            tc_mma<C::FMT>(tmem_d, a1, b0, idesc, 1u);  // Alo * Shi
        }
    }
}

__device__ __forceinline__ void tc_store_bf16x2(__nv_bfloat16* p, int64_t plane, int64_t idx, float v) {
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    p[idx] = hi;
    p[plane + idx] = __float2bfloat16_rn(v - __bfloat162float(hi));
}

// Epilogue of one 128 x width tile by the epilogue warp(s) of TMEM lane quarter `quarter`
// (chunks c0, c0 + cstep, ... of 32 columns each): read the accumulator and store it transposed,
// out[(l, n)][r], straight from the registers: lane = accumulator row r, so each store
// instruction writes 32 consecutive elements of one output row.  Every lane of the warp calls
// it (tcgen05.ld is warp-collective); `valid` false skips the stores.  G2 divides by
// ex[r] + ey[n] - lam[l] (row term per lane, column term shuffled from the lane that loaded
// it, loaded before the accumulator is read); G4 adds to psi_hat when `accumulate` is set
// (refinement).  `rowterm` is tc_rowterm's value for this lane.
template <int PASS>
__device__ __forceinline__ void tc_epilogue(const TcTile& T, void* Cv, int c_fmt, int accumulate, uint32_t tmem_acc,
                                            int quarter, int lane, bool valid, float rowterm, int c0 = 0,
                                            int cstep = 1) {
    const TcGeom& g = T.g;
    const int Mtot = g.Mtot, Mb = g.Mb, ldo = g.ldo;
    const int Nn = g.Nn;                      // columns of the pass (layer stride of the output)
    const int n0 = T.n0;
    const int nend = min(Nn, n0 + T.width);   // this tile's columns end here
    const int64_t cplane = g.cplane;
    const int m = T.m0 + quarter * 32 + lane;
    const bool row_ok = valid && m < Mtot;
    const int l = m < Mtot ? m / Mb : 0;
    const int r = m - l * Mb;
    float* Cf = static_cast<float*>(Cv) + g.cbase;
    __nv_bfloat16* Cb = static_cast<__nv_bfloat16*>(Cv) + g.cbase;
    const int64_t obase = (int64_t)l * Nn * ldo + r;
    for (int c = c0; c < (TC_BN + 31) / 32; c += cstep) {
        const int nb = n0 + c * 32;
        if (!valid || nb >= nend) break;  // warp-uniform (and the same for every epilogue warp)
        float eyl = 1.f;
        if constexpr (PASS == G2_FWD_Y) eyl = nb + lane < nend ? T.ey[nb + lane] : 1.f;
        uint32_t v[32];
        const uint32_t taddr = tmem_acc + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(c * 32);
        QG_LD32(v, taddr);
        asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
        if constexpr (PASS == G2_FWD_Y) {
            // spectral divide: the fast division is exact to ~2 ulp, far inside the BF16x3 /
            // TF32 error of the transform itself
#pragma unroll
            for (int j = 0; j < 32; ++j)
                v[j] = __float_as_uint(__fdividef(__uint_as_float(v[j]), rowterm + __shfl_sync(0xffffffffu, eyl, j)));
        }
        if (!row_ok) continue;
        const int ncol = min(32, nend - nb);
        const int64_t o0 = obase + (int64_t)nb * ldo;
        if (c_fmt == FMT_F32) {
            float* q = Cf + o0;
            if (ncol == 32) {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    float x = __uint_as_float(v[j]);
                    if (PASS == G4_INV_Y && accumulate) x += q[(int64_t)j * ldo];
                    q[(int64_t)j * ldo] = x;
                }
            } else {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    if (j >= ncol) break;
                    float x = __uint_as_float(v[j]);
                    if (PASS == G4_INV_Y && accumulate) x += q[(int64_t)j * ldo];
                    q[(int64_t)j * ldo] = x;
                }
            }
        } else {
            __nv_bfloat16* q = Cb + o0;
            if (ncol == 32) {
#pragma unroll
                for (int j = 0; j < 32; ++j) tc_store_bf16x2(q, cplane, (int64_t)j * ldo, __uint_as_float(v[j]));
            } else {
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    if (j >= ncol) break;
                    tc_store_bf16x2(q, cplane, (int64_t)j * ldo, __uint_as_float(v[j]));
                }
            }
        }
    }
}

}  // namespace qg
