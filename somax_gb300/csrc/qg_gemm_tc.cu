// Tensor-core DST-I GEMMs for sm_103a (5th-generation tensor cores), one output tile per CTA.
//
// C = A * S for one 128 x 128 output tile per CTA: A rows (layer, r) and S rows are both
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
#include <cstring>

#include "qg_tc.cuh"

namespace qg {

namespace {

constexpr int NTHREADS = 192;

template <int PREC>
__host__ __device__ constexpr int smem_bytes() {
    return TcCfg<PREC>::STAGES * tc_stage_bytes<PREC>() + TC_EPI_SMEM + 1024;
}

template <int PREC, int PASS>
__global__ void __launch_bounds__(NTHREADS, 1) k_gemm_tc(GemmArgs ga, const TcMaps* __restrict__ maps) {
    using C = TcCfg<PREC>;
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
    const TcGeom g = tc_geom<PASS>(M, ga.xplane, ga.yplane);
    const int m0 = t.mt * TC_BM, n0 = t.nt * TC_BN;
    const int nkb = (g.K + C::BK - 1) / C::BK;

    if (threadIdx.x == 0) {
        for (int s = 0; s < C::STAGES; ++s) {
            mbar_init(&full_bar[s], 1);
            mbar_init(&empty_bar[s], 1);
        }
        mbar_init(&acc_bar, 1);
        abort_flag = 0;
        n_issued = n_consumed = 0;
        mbar_init_fence();
    }
    if (warp == 1) tc_alloc(&tmem_slot, TC_BN);
    if (threadIdx.x == 32) {
        for (int a = 0; a < C::NA; ++a) tma_prefetch_desc(&tm->a[a]);
        for (int b = 0; b < C::NB; ++b) tma_prefetch_desc(&tm->b[b]);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
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
                uint8_t* st = smem + s * tc_stage_bytes<PREC>();
                mbar_expect_tx(&full_bar[s], tc_stage_bytes<PREC>());
                const int kx = kb * C::BK;
                for (int a = 0; a < C::NA; ++a) tma_load_2d(st + a * tc_tile_a_bytes<PREC>(), &tm->a[a], &full_bar[s], kx, m0);
                for (int b = 0; b < C::NB; ++b)
                    tma_load_2d(st + C::NA * tc_tile_a_bytes<PREC>() + b * tc_tile_b_bytes<PREC>(), &tm->b[b],
                                &full_bar[s], kx, n0);
                n_issued = kb + 1;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            for (int kb = 0; kb < nkb; ++kb) {
                const int s = kb % C::STAGES;
                if (!mbar_wait(&full_bar[s], (kb / C::STAGES) & 1, abort)) break;
                tc_fence_after();
                const uint32_t sa = su32(smem + s * tc_stage_bytes<PREC>());
                tc_mma_kblock<PREC>(tmem, sa, sa + C::NA * tc_tile_a_bytes<PREC>(), kb == 0);
                tc_commit(&empty_bar[s]);
                n_consumed = kb + 1;
            }
            tc_commit(&acc_bar);  // fires once every MMA issued above has completed
        }
    } else {
        // the accumulator barrier is committed even after an abort, so this wait also drains
        // the MMAs in flight before TMEM is read and freed
        const bool have = mbar_drain(&acc_bar, 0) && !*abort;
        tc_fence_after();
        float* stage = reinterpret_cast<float*>(smem + C::STAGES * tc_stage_bytes<PREC>()) + (warp - 2) * TC_STAGE_FLOATS;
        tc_epilogue<PASS>(M, g, ga.C, ga.c_fmt, ga.accumulate, m0, n0, tmem, warp & 3, lane, have, stage);
    }
    tc_fence_before();
    __syncthreads();
    if (abort_flag && threadIdx.x == 0) {
        // wait (bounded) for TMA copies that were issued but never consumed
        for (int kb = n_consumed; kb < n_issued; ++kb)
            mbar_drain(&full_bar[kb % C::STAGES], (kb / C::STAGES) & 1);
    }
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tc_dealloc(tmem, TC_BN);
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

int gemm_tc_tile_n(int) { return TC_BN; }

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
    cudaError_t e = encode(&tm.a[0], A, K, M.nl * Mb, pitch, prec, TC_BM);
    if (!e && prec == QG_DST_BF16X3) e = encode(&tm.a[1], A + a_plane_elems * es, K, M.nl * Mb, pitch, prec, TC_BM);
    // S of the contracted axis: K x K, pitch = the same axis' padded length
    const void* S = prec == QG_DST_BF16X3 ? (const void*)(xin ? M.Sx_bf : M.Sy_bf) : (const void*)(xin ? M.Sx : M.Sy);
    if (!e) e = encode(&tm.b[0], S, K, K, pitch, prec, TC_BN);
    if (!e && prec == QG_DST_BF16X3)
        e = encode(&tm.b[1], static_cast<const char*>(S) + (int64_t)K * pitch * es, K, K, pitch, prec, TC_BN);
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
