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
// The one-pass GEMM launch runs sixteen epilogue warps (warps 4-19, four per TMEM lane
// quarter, each draining every fourth 32-column chunk): the drain of a tile, not its loads or
// MMAs, bounds the pass when the stores split BF16 hi/lo or divide.  640 threads leave 96
// registers a thread, which the drain fits without spills.
constexpr int GEMM_EPI_WARPS = 16;
constexpr int PT_GEMM = 128 + 32 * GEMM_EPI_WARPS;
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

// Grid-wide barrier with a spin bounded by `wait` clock64 cycles.  Returns false (and flags the
// abort) on timeout or when this CTA already aborted.  A CTA that gives up leaves its arrival
// in *count, so the host zeroes both words before the next launch.
__device__ bool grid_sync(unsigned* count, unsigned* gen, int* flags, volatile int* abort, long long wait) {
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
                    if (clock64() - t0 > wait) {
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

template <int PREC, int PASS, int EPI = 4>
__device__ void gemm_phase(const PersistArgs& a, uint8_t* smem, Shared& sh, uint32_t tmem, Counters& c) {
    using C = TcCfg<PREC>;
    constexpr bool xin = pass_xin(PASS);
    const GemmTile* tiles = xin ? a.gx : a.gy;
    const int n = xin ? a.n_gx : a.n_gy;
    void* Cv = PASS == G1_FWD_X ? a.YA : PASS == G2_FWD_Y ? a.XB : PASS == G3_INV_X ? a.YB : (void*)a.XC;
    const int c_fmt = PASS == G4_INV_Y ? FMT_F32 : a.op_fmt;
    const TcMaps* maps = static_cast<const TcMaps*>(a.tc_maps);
    volatile int* abort = &sh.abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    if (warp == 0 && lane == 0) {
        proxy_fence_shared();  // the stencil phase wrote this shared memory with generic stores
        for (int t = blockIdx.x; t < n && !*abort; t += gridDim.x) {
            const GemmTile tl = tiles[t];
            if (tl.member < 0) continue;  // a padding entry of the balanced schedule
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
                                &sh.full[s], kb * C::BK, tl.nt * a.tile_n);
                sh.issued = (int)++c.prod_kb;
            }
        }
    } else if (warp == 1 && lane == 0) {
        for (int t = blockIdx.x; t < n && !*abort; t += gridDim.x) {
            const GemmTile tl = tiles[t];
            if (tl.member < 0) continue;  // a padding entry of the balanced schedule
            const TcGeom g = tc_geom<PASS>(a.members[tl.member], a.xplane, a.yplane);
            const int nkb = (g.K + C::BK - 1) / C::BK;
            const uint32_t buf = c.mma_tiles & 1, use = c.mma_tiles >> 1;
            if (!mbar_wait(&sh.tempty[buf], (use & 1) ^ 1, abort)) break;
            tc_fence_after();
            const uint32_t acc = tmem + buf * TC_TMEM_BUF;
            const int width = tc_tile_width(g.Nn, tl.nt, a.tile_n);
            for (int kb = 0; kb < nkb; ++kb) {
                const int s = c.mma_kb % C::STAGES;
                if (!mbar_wait(&sh.full[s], (c.mma_kb / C::STAGES) & 1, abort)) break;
                tc_fence_after();
                const uint32_t sa = su32(smem + s * tc_stage_bytes<PREC>());
                const int ksteps = (min(C::BK, g.K - kb * C::BK) + C::UMMA_K - 1) / C::UMMA_K;
                tc_mma_kblock<PREC>(acc, sa, sa + C::NA * tc_tile_a_bytes<PREC>(), kb == 0, ksteps, width);
                tc_commit(&sh.empty[s]);
                sh.consumed = (int)++c.mma_kb;
            }
            tc_commit(&sh.tfull[buf]);
            sh.committed = (int)++c.mma_tiles;
        }
    } else if (warp >= 4 && warp < 4 + EPI) {
        const int part = (warp - 4) >> 2;  // column chunks part, part + EPI / 4, ...
        const int step = gridDim.x;
        // Two-deep software pipeline over the CTA's tiles: the schedule entry two tiles ahead
        // and the next tile's member geometry load while the current tile drains, so that a
        // drain never starts with a chain of dependent global loads.
        int t = blockIdx.x;
        GemmTile ahead = t + step < n ? tiles[t + step] : GemmTile{-1, 0, 0};
        TcTile nxt = t < n ? tc_tile<PASS>(a.members, tiles[t], a.xplane, a.yplane, a.tile_n) : TcTile{};
        for (; t < n; t += step) {
            const TcTile tl = nxt;
            if (t + step < n) nxt = tc_tile<PASS>(a.members, ahead, a.xplane, a.yplane, a.tile_n);
            if (t + 2 * step < n) ahead = tiles[t + 2 * step];
            if (tl.member < 0) continue;  // a padding entry of the balanced schedule
            const float rowterm = tc_rowterm<PASS>(tl, warp & 3, lane);
            const uint32_t buf = c.epi_tiles & 1, use = c.epi_tiles >> 1;
            const bool have = mbar_wait(&sh.tfull[buf], use & 1, abort);
            if (!have) break;
            tc_fence_after();
            tc_epilogue<PASS>(tl, Cv, c_fmt, PASS == G4_INV_Y ? a.g4_accumulate : 0, tmem + buf * TC_TMEM_BUF,
                              warp & 3, lane, true, rowterm, part, EPI / 4);
            tc_fence_before();
            mbar_arrive(&sh.tempty[buf]);
            ++c.epi_tiles;
        }
    }
}

// Stencil tiles of one launch or phase, round-robin over the CTAs; with two box buffers the
// next tile's TMA copies run while the current tile is computed.  `sa` selects the input
// stage plane (q_sel), the mode (rhs / step) and the outputs.
template <class T>
__device__ void stencil_tiles(const StencilArgs& sa, int n_st, uint8_t* smem, size_t slot_bytes, size_t lap_offset,
                              int nbuf, Shared& sh, Counters& c) {
    using namespace st;
    const StencilMaps* maps = static_cast<const StencilMaps*>(sa.maps);
    float* sl = reinterpret_cast<float*>(smem + lap_offset);
    auto issue = [&](int t, int b) {
        const StencilTile tl = sa.tiles[t];
        const int nl = sa.members[tl.member].nl;
        float* sq = reinterpret_cast<float*>(smem + b * slot_bytes);
        proxy_fence_shared();  // generic accesses of this buffer finished before TMA rewrites it
        tile_issue<T>(&maps[tl.member], sa.q_sel, nl, tl.ty, tl.tx, sq, sq + nl * T::BOX, &sh.sbar[b]);
    };
    if (nbuf == 2 && threadIdx.x == 0 && (int)blockIdx.x < n_st) issue(blockIdx.x, 0);
    bool bad = false;
    for (int u = 0;; ++u) {
        const int t = blockIdx.x + u * gridDim.x;
        if (t >= n_st || sh.abort) break;
        const int b = nbuf == 2 ? (u & 1) : 0;
        if (threadIdx.x == 0) {
            if (nbuf == 1) {
                issue(t, 0);
            } else if (t + (int)gridDim.x < n_st) {
                issue(t + gridDim.x, b ^ 1);
            }
        }
        const StencilTile tl = sa.tiles[t];
        load_member(&sh.M, sa.members + tl.member);
        const bool need_lap = sa.params[(int64_t)tl.member * QG_NPARAMS + QG_P_NU4] != 0.f;
        __syncthreads();
        const bool have = mbar_wait(&sh.sbar[b], c.st_use[b] & 1, &sh.abort);
        ++c.st_use[b];
        float* sq = reinterpret_cast<float*>(smem + b * slot_bytes);
        float* sp = sq + sh.M.nl * T::BOX;
        bad |= stencil_tile<T>(sa, sh.M, tl, sq, sp, sl, sa.apply_bc, need_lap) || !have;
        __syncthreads();
    }
    if (bad && sa.flags) atomicOr(sa.flags, 1);
    // a prefetch issued for a tile beyond an abort is drained before the buffers are reused
    if (sh.abort && threadIdx.x == 0) {
        for (int b = 0; b < nbuf; ++b) mbar_drain(&sh.sbar[b], c.st_use[b] & 1);
    }
}

// Stencil phase of stage `k` of the persistent kernel.
template <class T>
__device__ void stencil_phase(const PersistArgs& a, int k, uint8_t* smem, Shared& sh, Counters& c) {
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
    stencil_tiles<T>(sa, a.n_st, smem, a.slot_bytes, a.lap_offset, a.st_nbuf, sh, c);
}

__device__ void init_shared(Shared& sh, int stages, int epi_warps = 4) {
    if (threadIdx.x == 0) {
        for (int s = 0; s < stages; ++s) {
            mbar_init(&sh.full[s], 1);
            mbar_init(&sh.empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&sh.tfull[b], 1);
            mbar_init(&sh.tempty[b], epi_warps * 32);  // every epilogue thread arrives
            mbar_init(&sh.sbar[b], 1);
        }
        sh.abort = 0;
        sh.issued = sh.consumed = sh.committed = 0;
        mbar_init_fence();
    }
}

// After an abort: drain TMA copies issued but not consumed, then the MMAs of the last
// committed accumulator, so that shared memory and TMEM are quiet before the CTA exits.
template <int STAGES>
__device__ void drain_after_abort(Shared& sh) {
    if (sh.abort && threadIdx.x == 0) {
        for (int kb = sh.consumed; kb < sh.issued; ++kb) mbar_drain(&sh.full[kb % STAGES], (kb / STAGES) & 1);
        if (sh.committed > 0) {
            const int t = sh.committed - 1;
            mbar_drain(&sh.tfull[t & 1], (t >> 1) & 1);
        }
    }
}

// One DST-I GEMM pass as its own launch: output tiles of all members round-robin over
// min(tiles, SMs) CTAs, two TMEM accumulators so a tile's epilogue overlaps the next
// tile's MMAs.
template <int PREC, int PASS>
__global__ void __launch_bounds__(PT_GEMM, 1) k_gemm_mt(PersistArgs a) {
    using C = TcCfg<PREC>;
    extern __shared__ uint8_t smem_raw[];
    __shared__ Shared sh;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    init_shared(sh, C::STAGES, GEMM_EPI_WARPS);
    if ((threadIdx.x >> 5) == 1) tc_alloc(&sh.tmem_slot, TC_TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh.tmem_slot;
    pdl_wait();
    pdl_launch_dependents();
    Counters c;
    gemm_phase<PREC, PASS, GEMM_EPI_WARPS>(a, smem, sh, tmem, c);
    __syncthreads();
    drain_after_abort<C::STAGES>(sh);
    tc_fence_before();
    __syncthreads();
    if ((threadIdx.x >> 5) == 1) {
        tc_fence_after();
        tc_dealloc(tmem, TC_TMEM_COLS);
    }
    if (threadIdx.x == 0 && sh.abort && a.flags) atomicOr(a.flags, 2);
}

// The RHS stencil as its own launch: tiles round-robin, double-buffered TMA boxes.
template <class T>
__global__ void __launch_bounds__(PT, 3) k_stencil_mt(StencilArgs sa, int n_st, size_t slot_bytes, size_t lap_offset,
                                                      int nbuf) {
    extern __shared__ uint8_t smem_raw[];
    __shared__ Shared sh;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    init_shared(sh, 0);
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();
    Counters c;
    stencil_tiles<T>(sa, n_st, smem, slot_bytes, lap_offset, nbuf, sh, c);
}

template <int PREC, class T>
__global__ void __launch_bounds__(PT, 1) k_persistent(PersistArgs a) {
    using C = TcCfg<PREC>;
    extern __shared__ uint8_t smem_raw[];
    __shared__ Shared sh;
    uint8_t* smem = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int warp = threadIdx.x >> 5;
    init_shared(sh, C::STAGES);
    if (warp == 1) tc_alloc(&sh.tmem_slot, TC_TMEM_COLS);
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = sh.tmem_slot;
    Counters c;
    volatile int* abort = &sh.abort;

    for (int step = 0; step < a.n_steps; ++step) {
        for (int k = 0; k < a.n_stages; ++k) {
            gemm_phase<PREC, G1_FWD_X>(a, smem, sh, tmem, c);
            if (!grid_sync(a.bar_count, a.bar_gen, a.flags, abort, a.bar_wait)) goto done;
            gemm_phase<PREC, G2_FWD_Y>(a, smem, sh, tmem, c);
            if (!grid_sync(a.bar_count, a.bar_gen, a.flags, abort, a.bar_wait)) goto done;
            gemm_phase<PREC, G3_INV_X>(a, smem, sh, tmem, c);
            if (!grid_sync(a.bar_count, a.bar_gen, a.flags, abort, a.bar_wait)) goto done;
            gemm_phase<PREC, G4_INV_Y>(a, smem, sh, tmem, c);
            if (!grid_sync(a.bar_count, a.bar_gen, a.flags, abort, a.bar_wait)) goto done;
            stencil_phase<T>(a, k, smem, sh, c);
            if (!grid_sync(a.bar_count, a.bar_gen, a.flags, abort, a.bar_wait)) goto done;
        }
    }
done:
    __syncthreads();
    drain_after_abort<C::STAGES>(sh);
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tc_dealloc(tmem, TC_TMEM_COLS);
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
                                                  : (size_t)TcCfg<QG_DST_BF16X3>::STAGES * tc_stage_bytes<QG_DST_BF16X3>());
    const size_t sten = large ? stencil_layout<st::TileL>(max_nl, a) : stencil_layout<st::TileS>(max_nl, a);
    return std::max(gemm, sten) + 1024;
}

size_t stencil_mt_smem_bytes(int max_nl, int large, size_t* slot, size_t* lap_off, int* nbuf) {
    PersistArgs a{};
    const size_t b = large ? stencil_layout<st::TileL>(max_nl, &a) : stencil_layout<st::TileS>(max_nl, &a);
    if (slot) *slot = a.slot_bytes;
    if (lap_off) *lap_off = a.lap_offset;
    if (nbuf) *nbuf = a.st_nbuf;
    return b + 1024;
}

int stencil_mt_blocks_per_sm(int max_nl, int large) {
    int n = 0;
    const size_t smem = stencil_mt_smem_bytes(max_nl, large, nullptr, nullptr, nullptr);
    if (large)
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_stencil_mt<st::TileL>, PT, smem);
    else
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_stencil_mt<st::TileS>, PT, smem);
    return n > 0 ? n : 1;
}

cudaError_t launch_stencil_mt(const StencilArgs& sa, int n_st, int grid, int max_nl, int large, cudaStream_t s,
                              bool pdl) {
    size_t slot = 0, lap = 0;
    int nbuf = 1;
    const size_t smem = stencil_mt_smem_bytes(max_nl, large, &slot, &lap, &nbuf);
    if (large) return launch_k(k_stencil_mt<st::TileL>, grid, PT, smem, s, pdl, sa, n_st, slot, lap, nbuf);
    return launch_k(k_stencil_mt<st::TileS>, grid, PT, smem, s, pdl, sa, n_st, slot, lap, nbuf);
}

template <int PREC>
size_t gemm_mt_smem() {
    return (size_t)TcCfg<PREC>::STAGES * tc_stage_bytes<PREC>() + 1024;
}

cudaError_t launch_gemm_mt(const PersistArgs& a, int pass, int grid, int precision, cudaStream_t s, bool pdl) {
#define QG_GMT(P)                                                                                                  \
    switch (pass) {                                                                                                \
        case G1_FWD_X: return launch_k(k_gemm_mt<P, G1_FWD_X>, grid, PT_GEMM, gemm_mt_smem<P>(), s, pdl, a);          \
        case G2_FWD_Y: return launch_k(k_gemm_mt<P, G2_FWD_Y>, grid, PT_GEMM, gemm_mt_smem<P>(), s, pdl, a);          \
        case G3_INV_X: return launch_k(k_gemm_mt<P, G3_INV_X>, grid, PT_GEMM, gemm_mt_smem<P>(), s, pdl, a);          \
        case G4_INV_Y: return launch_k(k_gemm_mt<P, G4_INV_Y>, grid, PT_GEMM, gemm_mt_smem<P>(), s, pdl, a);          \
        default: return cudaErrorInvalidValue;                                                                     \
    }
    if (precision == QG_DST_TF32) { QG_GMT(QG_DST_TF32) }
    if (precision == QG_DST_BF16X3) { QG_GMT(QG_DST_BF16X3) }
#undef QG_GMT
    return cudaErrorInvalidValue;
}

cudaError_t persistent_init() {
    cudaError_t e = cudaSuccess;
#define QG_MTATTR(K, B)                                                                                       \
    if (!e) e = cudaFuncSetAttribute(K, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)(B));
    QG_MTATTR(k_stencil_mt<st::TileS>, stencil_mt_smem_bytes(kMaxLayers, 0, nullptr, nullptr, nullptr))
    QG_MTATTR(k_stencil_mt<st::TileL>, stencil_mt_smem_bytes(kMaxLayers, 1, nullptr, nullptr, nullptr))
    QG_MTATTR((k_gemm_mt<QG_DST_TF32, G1_FWD_X>), gemm_mt_smem<QG_DST_TF32>())
    QG_MTATTR((k_gemm_mt<QG_DST_TF32, G2_FWD_Y>), gemm_mt_smem<QG_DST_TF32>())
    QG_MTATTR((k_gemm_mt<QG_DST_TF32, G3_INV_X>), gemm_mt_smem<QG_DST_TF32>())
    QG_MTATTR((k_gemm_mt<QG_DST_TF32, G4_INV_Y>), gemm_mt_smem<QG_DST_TF32>())
    QG_MTATTR((k_gemm_mt<QG_DST_BF16X3, G1_FWD_X>), gemm_mt_smem<QG_DST_BF16X3>())
    QG_MTATTR((k_gemm_mt<QG_DST_BF16X3, G2_FWD_Y>), gemm_mt_smem<QG_DST_BF16X3>())
    QG_MTATTR((k_gemm_mt<QG_DST_BF16X3, G3_INV_X>), gemm_mt_smem<QG_DST_BF16X3>())
    QG_MTATTR((k_gemm_mt<QG_DST_BF16X3, G4_INV_Y>), gemm_mt_smem<QG_DST_BF16X3>())
#undef QG_MTATTR
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
