// Persistent time-step kernel: one cooperative launch advances every member of a plan by
// n_steps steps.  Each RK stage is five phases separated by grid barriers:
//
//   G1, G2, G3, G4   DST-I GEMM passes on the tensor cores (tcgen05), output tiles of all
//                    members dealt round-robin to the CTAs; per CTA warp 0 issues TMA, warp 1
//                    issues MMAs into one of two TMEM accumulators, warps 4-7 drain the other
//                    accumulator (epilogue overlaps the next tile's MMAs)
//   stencil          RHS + Shu-Osher stage update + next-stage layer->mode operand, tiles of
//                    all members round-robin, the next tile's TMA halo boxes loaded while the
//                    current one is computed
//
// One CTA per SM (up to the number of tiles), 256 threads.  The grid barrier is a counter +
// generation word in global memory with release/acquire ordering and a bounded spin; every
// mbarrier wait is bounded too.  On a timeout the kernel records bit 1 in the status word,
// stops issuing work, drains its copies and MMAs in flight and frees its TMEM.
#include <algorithm>

#include "qg_stencil_tile.cuh"
#include "qg_tc.cuh"

namespace qg {

namespace {

constexpr int PT = 256;  // threads per CTA (the stencil tile needs exactly 256)
static_assert(st::NTHREADS == PT, "stencil tile thread count");

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void red_release_add(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ void proxy_fence_global() { asm volatile("fence.proxy.async.global;" ::: "memory"); }
__device__ __forceinline__ void proxy_fence_shared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Grid-wide barrier with a bounded spin.  Returns false (and flags the abort) on timeout or
// when this CTA already aborted.
__device__ bool grid_sync(unsigned* count, unsigned* gen, int* flags, volatile int* abort) {
    __syncthreads();
    if (threadIdx.x == 0) {
        bool ok = !*abort;
        if (ok) {
            __threadfence();
            const unsigned g = ld_acquire(gen);  // cannot advance before this CTA arrives
            const unsigned arrived = atomicAdd(count, 1u);
            if (arrived == gridDim.x - 1) {
                atomicExch(count, 0u);
                __threadfence();
                red_release_add(gen, 1u);
            } else {
                const long long t0 = clock64();
                while (ld_acquire(gen) == g) {
                    if (clock64() - t0 > kTimeoutCycles) {
                        ok = false;
                        break;
                    }
                }
            }
        }
        if (!ok) {
            *abort = 1;
            if (flags) atomicOr(flags, 2);
        }
        __threadfence();
    }
    __syncthreads();
    proxy_fence_global();  // later TMA (async proxy) reads see what other CTAs wrote
    return !*abort;
}

struct Counters {
    uint32_t prod_kb = 0;   // k-blocks issued by the producer
    uint32_t mma_kb = 0;    // k-blocks consumed by the MMA thread
    uint32_t mma_tiles = 0; // accumulators filled
    uint32_t epi_tiles = 0; // accumulators drained
    uint32_t st_use[2] = {0, 0};  // stencil box loads per buffer
};

struct Shared {
    uint64_t full[4], empty[4], tfull[2], tempty[2], sbar[2];
    uint32_t tmem_slot;
    int abort;
    int issued, consumed, committed;  // for draining after an abort
    MemberDev M;                      // constants of the current stencil tile
};

template <int PREC, int PASS>
__device__ void gemm_phase(const PersistArgs& a, uint8_t* smem, Shared& sh, uint32_t tmem, Counters& c) {
    using C = TcCfg<PREC>;
    constexpr bool xin = (PASS == G1_FWD_X || PASS == G4_INV_X);
    const GemmTile* tiles = xin ? a.gx : a.gy;
    const int n = xin ? a.n_gx : a.n_gy;
    void* Cv = PASS == G1_FWD_X ? a.YA : PASS == G2_FWD_Y ? a.YB : PASS == G3_INV_Y ? a.XB : (void*)a.XC;
    const int c_fmt = PASS == G4_INV_X ? FMT_F32 : a.op_fmt;
    const TcMaps* maps = static_cast<const TcMaps*>(a.tc_maps);
    volatile int* abort = &sh.abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (warp == 0 && lane == 0) {
        proxy_fence_shared();  // the stencil phase wrote this shared memory with generic stores
        for (int t = blockIdx.x; t < n && !*abort; t += gridDim.x) {
            const GemmTile tl = tiles[t];
            const TcMaps* tm = maps + (tl.member * 4 + PASS);
            const TcGeom g = tc_geom<PASS>(a.members[tl.member], a.xplane, a.yplane);
            const int nkb = (g.K + C::BK - 1) / C::BK;
            for (int kb = 0; kb < nkb; ++kb) {
                const int s = c.prod_kb % C::STAGES;
                if (!mbar_wait(&sh.empty[s], ((c.prod_kb / C::STAGES) & 1) ^ 1, abort)) break;
                uint8_t* stg = smem + s * tc_stage_bytes<PREC>();
                mbar_expect_tx(&sh.full[s], tc_stage_bytes<PREC>());
                for (int q = 0; q < C::NA; ++q)
                    tma_load_2d(stg + q * tc_tile_a_bytes<PREC>(), &tm->a[q], &sh.full[s], kb * C::BK, tl.mt * TC_BM);
                for (int q = 0; q < C::NB; ++q)
                    tma_load_2d(stg + C::NA * tc_tile_a_bytes<PREC>() + q * tc_tile_b_bytes<PREC>(), &tm->b[q],
                                &sh.full[s], kb * C::BK, tl.nt * TC_BN);
                sh.issued = (int)++c.prod_kb;
            }
        }
    } else if (warp == 1 && lane == 0) {
        for (int t = blockIdx.x; t < n && !*abort; t += gridDim.x) {
            const GemmTile tl = tiles[t];
            const TcGeom g = tc_geom<PASS>(a.members[tl.member], a.xplane, a.yplane);
            const int nkb = (g.K + C::BK - 1) / C::BK;
            const uint32_t buf = c.mma_tiles & 1, use = c.mma_tiles >> 1;
            if (!mbar_wait(&sh.tempty[buf], (use & 1) ^ 1, abort)) break;
            tc_fence_after();
            const uint32_t acc = tmem + buf * TC_BN;
            for (int kb = 0; kb < nkb; ++kb) {
                const int s = c.mma_kb % C::STAGES;
                if (!mbar_wait(&sh.full[s], (c.mma_kb / C::STAGES) & 1, abort)) break;
                tc_fence_after();
                const uint32_t sa = su32(smem + s * tc_stage_bytes<PREC>());
                tc_mma_kblock<PREC>(acc, sa, sa + C::NA * tc_tile_a_bytes<PREC>(), kb == 0);
                tc_commit(&sh.empty[s]);
                sh.consumed = (int)++c.mma_kb;
            }
            tc_commit(&sh.tfull[buf]);
            sh.committed = (int)++c.mma_tiles;
        }
    } else if (warp >= 4) {
        for (int t = blockIdx.x; t < n; t += gridDim.x) {
            const GemmTile tl = tiles[t];
            const MemberDev& M = a.members[tl.member];
            const TcGeom g = tc_geom<PASS>(M, a.xplane, a.yplane);
            const uint32_t buf = c.epi_tiles & 1, use = c.epi_tiles >> 1;
            const bool have = mbar_wait(&sh.tfull[buf], use & 1, abort);
            if (!have) break;
            tc_fence_after();
            float* stage = reinterpret_cast<float*>(smem + C::STAGES * tc_stage_bytes<PREC>()) + (warp - 4) * TC_STAGE_FLOATS;
            tc_epilogue<PASS>(M, g, Cv, c_fmt, 0, tl.mt * TC_BM, tl.nt * TC_BN, tmem + buf * TC_BN, warp & 3, lane,
                              true, stage);
            tc_fence_before();
            mbar_arrive(&sh.tempty[buf]);
            ++c.epi_tiles;
        }
    }
}

// Stencil phase of stage `k`: tiles round-robin; with two box buffers the next tile's TMA
// copies run while the current tile is computed.
template <class T>
__device__ void stencil_phase(const PersistArgs& a, int k, uint8_t* smem, Shared& sh, Counters& c) {
    using namespace st;
    const StencilMaps* maps = static_cast<const StencilMaps*>(a.st_maps);
    const bool fin = (k == a.n_stages - 1);
    StencilArgs sa{};
    sa.members = a.members;
    sa.tiles = a.st;
    sa.maps = a.st_maps;
    sa.q_sel = k;
    sa.params = a.params;
    sa.apply_bc = 1;
    sa.xplane = a.xplane;
    sa.y0 = a.S[0];
    sa.y_next = fin ? a.S[0] : a.S[k + 1];
    sa.final_stage = fin;
    sa.a = a.sa[k];
    sa.b = a.sb[k];
    sa.dt = a.dt;
    sa.xa = a.XA;
    sa.xa_fmt = a.op_fmt;
    sa.xq = nullptr;
    sa.flags = a.flags;
    float* sl = reinterpret_cast<float*>(smem + a.lap_offset);
    const int nbuf = a.st_nbuf;

    auto issue = [&](int t, int b) {
        const StencilTile tl = a.st[t];
        const int nl = a.members[tl.member].nl;
        float* sq = reinterpret_cast<float*>(smem + b * a.slot_bytes);
        proxy_fence_shared();  // generic accesses of this buffer finished before TMA rewrites it
        tile_issue<T>(&maps[tl.member], k, nl, tl.ty, tl.tx, sq, sq + nl * T::BOX, &sh.sbar[b]);
    };
    if (nbuf == 2 && threadIdx.x == 0 && (int)blockIdx.x < a.n_st) issue(blockIdx.x, 0);
    bool bad = false;
    for (int u = 0;; ++u) {
        const int t = blockIdx.x + u * gridDim.x;
        if (t >= a.n_st || sh.abort) break;
        const int b = nbuf == 2 ? (u & 1) : 0;
        if (threadIdx.x == 0) {
            if (nbuf == 1) {
                issue(t, 0);
            } else if (t + (int)gridDim.x < a.n_st) {
                issue(t + gridDim.x, b ^ 1);
            }
        }
        const StencilTile tl = a.st[t];
        load_member(&sh.M, a.members + tl.member);
        const bool need_lap = a.params[(int64_t)tl.member * QG_NPARAMS + QG_P_NU4] != 0.f;
        __syncthreads();
        const bool have = mbar_wait(&sh.sbar[b], c.st_use[b] & 1, &sh.abort);
        ++c.st_use[b];
        float* sq = reinterpret_cast<float*>(smem + b * a.slot_bytes);
        float* sp = sq + sh.M.nl * T::BOX;
        stencil_fix_box<T>(sh.M, sq, sp, sl, tl.ty, tl.tx, 1, need_lap);
        __syncthreads();
        bad |= stencil_compute<T>(sa, sh.M, tl, sq, sp, sl) || !have;
        __syncthreads();
    }
    if (bad && a.flags) atomicOr(a.flags, 1);
    // a prefetch issued for a tile beyond an abort is drained before the buffers are reused
    if (sh.abort && threadIdx.x == 0) {
        for (int b = 0; b < nbuf; ++b) mbar_drain(&sh.sbar[b], c.st_use[b] & 1);
    }
}

template <int PREC, class T>
__global__ void __launch_bounds__(PT, 1) k_persistent(PersistArgs a) {
    using C = TcCfg<PREC>;
    extern __shared__ uint8_t smem_raw[];
    __shared__ Shared sh;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int s = 0; s < C::STAGES; ++s) {
            mbar_init(&sh.full[s], 1);
            mbar_init(&sh.empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&sh.tfull[b], 1);
            mbar_init(&sh.tempty[b], 4 * 32);  // every epilogue thread arrives
            mbar_init(&sh.sbar[b], 1);
        }
        sh.abort = 0;
        sh.issued = sh.consumed = sh.committed = 0;
        mbar_init_fence();
    }
    if (warp == 1) tc_alloc(&sh.tmem_slot, 2 * TC_BN);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh.tmem_slot;
    Counters c;
    volatile int* abort = &sh.abort;

    for (int step = 0; step < a.n_steps; ++step) {
        for (int k = 0; k < a.n_stages; ++k) {
            gemm_phase<PREC, G1_FWD_X>(a, smem, sh, tmem, c);
            if (!grid_sync(a.bar_count, a.bar_gen, a.flags, abort)) goto done;
            gemm_phase<PREC, G2_FWD_Y>(a, smem, sh, tmem, c);
            if (!grid_sync(a.bar_count, a.bar_gen, a.flags, abort)) goto done;
            gemm_phase<PREC, G3_INV_Y>(a, smem, sh, tmem, c);
            if (!grid_sync(a.bar_count, a.bar_gen, a.flags, abort)) goto done;
            gemm_phase<PREC, G4_INV_X>(a, smem, sh, tmem, c);
            if (!grid_sync(a.bar_count, a.bar_gen, a.flags, abort)) goto done;
            stencil_phase<T>(a, k, smem, sh, c);
            if (!grid_sync(a.bar_count, a.bar_gen, a.flags, abort)) goto done;
        }
    }
done:
    __syncthreads();
    if (*abort && threadIdx.x == 0) {
        // drain: TMA copies issued but not consumed, then the MMAs of the last committed tile
        for (int kb = sh.consumed; kb < sh.issued; ++kb)
            mbar_drain(&sh.full[kb % C::STAGES], (kb / C::STAGES) & 1);
        if (sh.committed > 0) {
            const int t = sh.committed - 1;
            mbar_drain(&sh.tfull[t & 1], (t >> 1) & 1);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tc_dealloc(tmem, 2 * TC_BN);
    }
}

}  // namespace

template <class T>
size_t stencil_layout(int max_nl, PersistArgs* a) {
    const size_t budget = 228 * 1024;  // dynamic shared memory left beside the static part
    const size_t slot = (st::tile_box_bytes<T>(max_nl) + 1023) & ~size_t(1023);
    const size_t lap = (st::tile_lap_bytes<T>(max_nl) + 1023) & ~size_t(1023);
    const int nbuf = (2 * slot + lap <= budget) ? 2 : 1;
    if (a) {
        a->slot_bytes = slot;
        a->lap_offset = nbuf * slot;
        a->st_nbuf = nbuf;
    }
    return nbuf * slot + lap;
}

size_t persistent_smem_bytes(int precision, int max_nl, int large, PersistArgs* a) {
    const size_t gemm = (precision == QG_DST_TF32 ? (size_t)TcCfg<QG_DST_TF32>::STAGES * tc_stage_bytes<QG_DST_TF32>()
                                                  : (size_t)TcCfg<QG_DST_BF16X3>::STAGES * tc_stage_bytes<QG_DST_BF16X3>()) +
                        TC_EPI_SMEM;
    const size_t sten = large ? stencil_layout<st::TileL>(max_nl, a) : stencil_layout<st::TileS>(max_nl, a);
    return std::max(gemm, sten) + 1024;
}

cudaError_t persistent_init() {
    cudaError_t e = cudaSuccess;
#define QG_PATTR(P, T, L)                                                                                      \
    if (!e)                                                                                                    \
        e = cudaFuncSetAttribute(k_persistent<P, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,              \
                                 (int)persistent_smem_bytes(P, kMaxLayers, L, nullptr));
    QG_PATTR(QG_DST_TF32, st::TileS, 0)
    QG_PATTR(QG_DST_TF32, st::TileL, 1)
    QG_PATTR(QG_DST_BF16X3, st::TileS, 0)
    QG_PATTR(QG_DST_BF16X3, st::TileL, 1)
#undef QG_PATTR
    return e;
}

cudaError_t launch_persistent(const PersistArgs& a, int grid, int precision, cudaStream_t s) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3(PT);
    cfg.dynamicSmemBytes = persistent_smem_bytes(precision, a.max_nl, a.st_large, nullptr);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;  // all CTAs co-resident: the grid barrier needs it
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (precision == QG_DST_TF32)
        return a.st_large ? cudaLaunchKernelEx(&cfg, k_persistent<QG_DST_TF32, st::TileL>, a)
                          : cudaLaunchKernelEx(&cfg, k_persistent<QG_DST_TF32, st::TileS>, a);
    if (precision == QG_DST_BF16X3)
        return a.st_large ? cudaLaunchKernelEx(&cfg, k_persistent<QG_DST_BF16X3, st::TileL>, a)
                          : cudaLaunchKernelEx(&cfg, k_persistent<QG_DST_BF16X3, st::TileS>, a);
    return cudaErrorInvalidValue;
}

}  // namespace qg
