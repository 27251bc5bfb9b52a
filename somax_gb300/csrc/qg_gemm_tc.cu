// Tensor-core DST-I GEMMs for sm_103a (5th-generation tensor cores).
//
// C = A * S for one 128 x BN output tile per CTA: A rows (layer, r) and S rows are both
// K-major, so both operands are fed to tcgen05.mma straight from 128-byte-swizzled shared
// memory that TMA fills; the FP32 accumulator lives in tensor memory (TMEM) and the
// epilogue warps read it back with tcgen05.ld and apply the pass's store (transposed,
// spectral divide, accumulate).
//
//   TF32   : kind::tf32, A and S read as float32 (the tensor core uses their top 19 bits)
//   BF16x3 : kind::f16 with bf16 operands split x = hi + lo; D += Ahi Shi + Ahi Slo + Alo Shi
//
// Warp roles (192 threads): warp 0 issues TMA, warp 1 owns TMEM and issues the MMAs,
// warps 2-5 are the epilogue (warp w reads TMEM lanes 32 (w % 4) .. + 31).  Every mbarrier
// wait is bounded (clock64); on timeout the kernel sets bit 1 of the plan's status word,
// stops issuing work, drains what it issued and frees its TMEM.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cudaTypedefs.h>

#include <cstring>

#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {

namespace {

constexpr int BM = 128;
constexpr int BN = 128;
constexpr int NTHREADS = 192;

struct TcMaps {
    CUtensorMap a[2];  // A hi (or f32), A lo
    CUtensorMap b[2];  // S hi (or f32), S lo
};
static_assert(sizeof(TcMaps) == kTcMapsBytes, "TcMaps size");

template <int PREC>
struct Cfg;
template <>
struct Cfg<QG_DST_TF32> {
    static constexpr int BK = 32;  // 32 fp32 = 128 B rows
    static constexpr int STAGES = 4;
    static constexpr int ESIZE = 4;
    static constexpr int NA = 1, NB = 1;           // operand planes
    static constexpr int UMMA_K = 8;               // 32 bytes per MMA along K
    static constexpr uint32_t FMT = 2;             // tf32
};
template <>
struct Cfg<QG_DST_BF16X3> {
    static constexpr int BK = 64;  // 64 bf16 = 128 B rows
    static constexpr int STAGES = 3;
    static constexpr int ESIZE = 2;
    static constexpr int NA = 2, NB = 2;
    static constexpr int UMMA_K = 16;
    static constexpr uint32_t FMT = 1;             // bf16
};

template <int PREC>
__host__ __device__ constexpr int tile_a_bytes() { return BM * Cfg<PREC>::BK * Cfg<PREC>::ESIZE; }
template <int PREC>
__host__ __device__ constexpr int tile_b_bytes() { return BN * Cfg<PREC>::BK * Cfg<PREC>::ESIZE; }
template <int PREC>
__host__ __device__ constexpr int stage_bytes() { return Cfg<PREC>::NA * tile_a_bytes<PREC>() + Cfg<PREC>::NB * tile_b_bytes<PREC>(); }
template <int PREC>
__host__ __device__ constexpr int smem_bytes() { return Cfg<PREC>::STAGES * stage_bytes<PREC>() + 1024; }

// ---- tcgen05 wrappers ----------------------------------------------------------------
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row groups
// 1024 bytes apart (SBO), descriptor version 1.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;            // leading byte offset (unused for swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;  // stride byte offset
    d |= (uint64_t)1 << 46;            // version
    d |= (uint64_t)2 << 61;            // SWIZZLE_128B
    return d;
}

template <uint32_t FMT>
__device__ __forceinline__ void mma(uint32_t tmem_d, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
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
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(su32(bar))
                 : "memory");
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

__device__ __forceinline__ void store_bf16x2(__nv_bfloat16* p, int64_t plane, int64_t idx, float v) {
    const __nv_bfloat16 hi = __float2bfloat16_rn(v);
    p[idx] = hi;
    p[plane + idx] = __float2bfloat16_rn(v - __bfloat162float(hi));
}

// ---- the kernel ------------------------------------------------------------------------
template <int PREC, int PASS>
__global__ void __launch_bounds__(NTHREADS, 1) k_gemm_tc(GemmArgs ga, const TcMaps* __restrict__ maps) {
    using C = Cfg<PREC>;
    extern __shared__ uint8_t smem_raw[];
    __shared__ __align__(8) uint64_t full_bar[C::STAGES];
    __shared__ __align__(8) uint64_t empty_bar[C::STAGES];
    __shared__ __align__(8) uint64_t acc_bar;
    __shared__ uint32_t tmem_slot;
    __shared__ int abort_flag;
    __shared__ int n_issued, n_consumed;

    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const GemmTile t = ga.tiles[blockIdx.x];
    const MemberDev& M = ga.members[t.member];
    const TcMaps* tm = maps + (t.member * 4 + PASS);

    const bool xin = (PASS == G1_FWD_X || PASS == G4_INV_X);
    const bool xout = (PASS == G3_INV_Y || PASS == G4_INV_X);
    const int Mb = xin ? M.Ny : M.Nx;
    const int K = xin ? M.Nx : M.Ny;
    const int Nn = K;
    const int Mtot = M.nl * Mb;
    const int m0 = t.mt * BM, n0 = t.nt * BN;
    const int nkb = (K + C::BK - 1) / C::BK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < C::STAGES; ++s) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&acc_bar, 1);
        abort_flag = 0;
        n_issued = n_consumed = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(&tmem_slot)),
                     "r"(BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    if (threadIdx.x == 32) {
        for (int a = 0; a < C::NA; ++a) tma_prefetch_desc(&tm->a[a]);
        for (int b = 0; b < C::NB; ++b) tma_prefetch_desc(&tm->b[b]);
    }
    fence_before();
    __syncthreads();
    fence_after();
    const uint32_t tmem = tmem_slot;
    volatile int* abort = &abort_flag;
    pdl_wait();
    pdl_launch_dependents();

    if (warp == 0) {
        if (lane == 0) {
            for (int kb = 0; kb < nkb; ++kb) {
                const int s = kb % C::STAGES;
                const uint32_t ph = (kb / C::STAGES) & 1;
                if (!mbar_wait(&empty_bar[s], ph ^ 1, abort)) break;
                uint8_t* st = smem + s * stage_bytes<PREC>();
                mbar_expect_tx(&full_bar[s], stage_bytes<PREC>());
                const int kx = kb * C::BK;
                for (int a = 0; a < C::NA; ++a) tma_load_2d(st + a * tile_a_bytes<PREC>(), &tm->a[a], &full_bar[s], kx, m0);
                for (int b = 0; b < C::NB; ++b)
                    tma_load_2d(st + C::NA * tile_a_bytes<PREC>() + b * tile_b_bytes<PREC>(), &tm->b[b], &full_bar[s], kx, n0);
                n_issued = kb + 1;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            const uint32_t idesc = (1u << 4) | (C::FMT << 7) | (C::FMT << 10) | ((uint32_t)(BN >> 3) << 17) |
                                   ((uint32_t)(BM >> 4) << 24);
            bool ok = true;
            for (int kb = 0; kb < nkb && ok; ++kb) {
                const int s = kb % C::STAGES;
                const uint32_t ph = (kb / C::STAGES) & 1;
                if (!mbar_wait(&full_bar[s], ph, abort)) {
                    ok = false;
                    break;
                }
                fence_after();
                const uint32_t sa = su32(smem + s * stage_bytes<PREC>());
                const uint32_t sb = sa + C::NA * tile_a_bytes<PREC>();
#pragma unroll
                for (int k = 0; k < C::BK / C::UMMA_K; ++k) {
                    const uint32_t koff = k * C::UMMA_K * C::ESIZE;  // 32 bytes per step
                    const uint64_t a0 = sdesc(sa + koff), b0 = sdesc(sb + koff);
                    const uint32_t acc0 = (kb > 0 || k > 0) ? 1u : 0u;
                    mma<C::FMT>(tmem, a0, b0, idesc, acc0);
                    if constexpr (C::NA == 2) {
                        const uint64_t a1 = sdesc(sa + tile_a_bytes<PREC>() + koff);
                        const uint64_t b1 = sdesc(sb + tile_b_bytes<PREC>() + koff);
                        mma<C::FMT>(tmem, a0, b1, idesc, 1u);  // Ahi * Slo
                        mma<C::FMT>(tmem, a1, b0, idesc, 1u);  // Alo * Shi
                    }
                }
                mma_commit(&empty_bar[s]);
                n_consumed = kb + 1;
            }
            mma_commit(&acc_bar);  // fires once every MMA issued above has completed
        }
    } else {
        // epilogue warps 2..5
        const int quarter = warp & 3;
        const int rl = quarter * 32 + lane;
        const int m = m0 + rl;
        // the accumulator barrier is committed even after an abort, so this wait also drains
        // the MMAs in flight before TMEM is read and freed
        const bool have = mbar_drain(&acc_bar, 0) && !*abort;
        fence_after();
        const int l = m < Mtot ? m / Mb : 0;
        const int r = m - l * Mb;
        const int ldo = xout ? M.Px : M.Py;
        const int64_t cbase = xout ? M.off_x : M.off_y;
        const int64_t cplane = xout ? ga.xplane : ga.yplane;
        const float exr = (PASS == G2_FWD_Y && m < Mtot) ? M.ex[r] : 0.f;
        const float laml = M.lam[l];
        float* Cf = static_cast<float*>(ga.C) + cbase;
        __nv_bfloat16* Cb = static_cast<__nv_bfloat16*>(ga.C) + cbase;
        for (int c = 0; c < BN / 32; ++c) {
            uint32_t v[32];
            const uint32_t taddr = tmem + ((uint32_t)(quarter * 32) << 16) + (uint32_t)(c * 32);
            QG_LD32(v, taddr);
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (!have || m >= Mtot) continue;
            const int nb = n0 + c * 32;
            if (nb >= Nn) continue;
            if constexpr (PASS == G1_FWD_X || PASS == G3_INV_Y) {
                // transposed store: out[(l, n)][r]; lanes hold consecutive r -> coalesced
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    if (nb + j >= Nn) break;
                    const float x = __uint_as_float(v[j]);
                    const int64_t o = ((int64_t)l * Nn + nb + j) * ldo + r;
                    if (ga.c_fmt == FMT_F32)
                        Cf[o] = x;
                    else
                        store_bf16x2(Cb, cplane, o, x);
                }
            } else {
                const int64_t o = (int64_t)m * ldo + nb;
#pragma unroll
                for (int j = 0; j < 32; ++j) {
                    if (nb + j >= Nn) break;
                    float x = __uint_as_float(v[j]);
                    if constexpr (PASS == G2_FWD_Y) x = x / (exr + M.ey[nb + j] - laml);
                    if (ga.c_fmt == FMT_F32) {
                        if (PASS == G4_INV_X && ga.accumulate) x += Cf[o + j];
                        Cf[o + j] = x;
                    } else {
                        store_bf16x2(Cb, cplane, o + j, x);
                    }
                }
            }
        }
    }
    fence_before();
    __syncthreads();
    if (abort_flag && threadIdx.x == 0) {
        // wait (bounded) for TMA copies that were issued but never consumed
        for (int kb = n_consumed; kb < n_issued; ++kb)
            mbar_drain(&full_bar[kb % C::STAGES], (kb / C::STAGES) & 1);
    }
    __syncthreads();
    if (warp == 1) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN));
    }
    if (threadIdx.x == 0 && abort_flag && ga.flags) atomicOr(ga.flags, 2);
}

template <int PREC>
cudaError_t set_attrs() {
    cudaError_t e = cudaSuccess;
#define QG_ATTR(P)                                                                                         \
    if (!e)                                                                                                \
        e = cudaFuncSetAttribute(k_gemm_tc<PREC, P>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes<PREC>());
    QG_ATTR(G1_FWD_X) QG_ATTR(G2_FWD_Y) QG_ATTR(G3_INV_Y) QG_ATTR(G4_INV_X)
#undef QG_ATTR
    return e;
}

template <int PREC>
cudaError_t launch(const GemmArgs& g, int ntiles, cudaStream_t s, bool pdl) {
    const TcMaps* maps = static_cast<const TcMaps*>(g.tc_maps);
    const int sm = smem_bytes<PREC>();
    switch (g.pass) {
        case G1_FWD_X: return launch_k(k_gemm_tc<PREC, G1_FWD_X>, ntiles, NTHREADS, sm, s, pdl, g, maps);
        case G2_FWD_Y: return launch_k(k_gemm_tc<PREC, G2_FWD_Y>, ntiles, NTHREADS, sm, s, pdl, g, maps);
        case G3_INV_Y: return launch_k(k_gemm_tc<PREC, G3_INV_Y>, ntiles, NTHREADS, sm, s, pdl, g, maps);
        case G4_INV_X: return launch_k(k_gemm_tc<PREC, G4_INV_X>, ntiles, NTHREADS, sm, s, pdl, g, maps);
        default: return cudaErrorInvalidValue;
    }
}

// 2-D tensor map over `rows` rows of `cols` valid elements with a row pitch of `pitch`
// elements; columns >= cols and rows >= rows read as zero.  128-byte rows, 128-byte swizzle.
cudaError_t encode(CUtensorMap* m, const void* base, int cols, int rows, int pitch, int prec, int box_rows) {
    const bool bf = prec == QG_DST_BF16X3;
    const int es = bf ? 2 : 4;
    const uint64_t dims[2] = {(uint64_t)cols, (uint64_t)rows};
    const uint64_t strides[1] = {(uint64_t)pitch * es};
    const uint32_t box[2] = {(uint32_t)(128 / es), (uint32_t)box_rows};
    return tmap_encode(m, bf ? 1 : 0, 2, base, dims, strides, box, 1);
}

}  // namespace

cudaError_t gemm_tc_init() {
    int dev = 0, major = 0, minor = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (!e) e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    if (!e) e = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (e) return e;
    if (major != 10 || minor != 3) return cudaErrorNotSupported;  // built for sm_103a only
    if (!e) e = set_attrs<QG_DST_TF32>();
    if (!e) e = set_attrs<QG_DST_BF16X3>();
    return e;
}

int gemm_tc_tile_n(int) { return BN; }

// Tensor maps of one member for one pass: A from the pass's input plane(s), S of the
// contracted axis.  `a_plane` is the plane base (all members), `a_plane_elems` its size.
cudaError_t gemm_tc_encode(const MemberDev& M, int pass, const void* a_plane, int64_t a_plane_elems, int prec,
                           void* out) {
    TcMaps tm;
    std::memset(&tm, 0, sizeof(tm));
    const bool xin = (pass == G1_FWD_X || pass == G4_INV_X);
    const int Mb = xin ? M.Ny : M.Nx, K = xin ? M.Nx : M.Ny, pitch = xin ? M.Px : M.Py;
    const int64_t off = xin ? M.off_x : M.off_y;
    const int es = prec == QG_DST_BF16X3 ? 2 : 4;
    const char* A = static_cast<const char*>(a_plane) + off * es;
    cudaError_t e = encode(&tm.a[0], A, K, M.nl * Mb, pitch, prec, BM);
    if (!e && prec == QG_DST_BF16X3) e = encode(&tm.a[1], A + a_plane_elems * es, K, M.nl * Mb, pitch, prec, BM);
    // S of the contracted axis: K x K, pitch = the same axis' padded length
    const void* S = prec == QG_DST_BF16X3 ? (const void*)(xin ? M.Sx_bf : M.Sy_bf) : (const void*)(xin ? M.Sx : M.Sy);
    if (!e) e = encode(&tm.b[0], S, K, K, pitch, prec, BN);
    if (!e && prec == QG_DST_BF16X3)
        e = encode(&tm.b[1], static_cast<const char*>(S) + (int64_t)K * pitch * es, K, K, pitch, prec, BN);
    if (!e) std::memcpy(out, &tm, sizeof(tm));
    return e;
}

cudaError_t launch_gemm_tc(const GemmArgs& g, int ntiles, int precision, cudaStream_t s, bool pdl) {
    if (!g.tc_maps) return cudaErrorInvalidValue;
    if (precision == QG_DST_TF32) return launch<QG_DST_TF32>(g, ntiles, s, pdl);
    if (precision == QG_DST_BF16X3) return launch<QG_DST_BF16X3>(g, ntiles, s, pdl);
    return cudaErrorInvalidValue;
}

}  // namespace qg
