// The fused RHS stencil as a warp column sweep (the multi-launch path's stencil).
//
// One warp owns a strip of 32 columns: lanes 2..29 produce the 28 output columns
// x0 .. x0 + 27 and lanes 0, 1, 30, 31 are the halo (the biharmonic term reaches two cells).
// The warp walks down a block of rows with every layer's q, psi (mixed from psi_hat on the
// fly, Cm2l) and lap(q) in four-row register windows; east / west neighbours come from the
// adjacent lanes by warp shuffles when they are used, north / south from the windows.  Every input element is
// read once per strip with coalesced row loads issued two rows ahead of their use; nothing
// goes through shared memory and nothing synchronises beyond the warp.
//
// Per row (arrays relative to the member, BC = zero ring of q when apply_bc):
//   ingest(r): q(r), psi_hat(r) -> q, psi = Z Cm2l psi_hat, east / west copies, lap q(r - 1)
//   output(r - 2): Arakawa J(psi, q) + beta term, wind, drag, nu lap q, nu4 lap(lap q),
//                  then the Shu-Osher stage update and the next stage's Cl2m operand (step
//                  mode) or dq (rhs mode), as the tile stencil (qg_stencil_tile.cuh) does.
#include <cuda_bf16.h>

#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {

namespace {

constexpr int kLanes = 32;
constexpr int kHalo = 2;
constexpr int kOut = kLanes - 2 * kHalo;  // 28 output columns per strip
constexpr int kWarps = 4;                 // warps per CTA (independent strips)

struct Coef {
    float nu, kappa, tau0, nu4;
    float idx2, idy2, i12, b12;
    float invH0;
};

template <int NL>
struct Win {
    // four-row windows indexed by row & 3 (east / west values come from the neighbouring
    // lanes when they are used, which keeps the windows small enough for 16 warps per SM)
    float q[NL][4], p[NL][4], lq[NL][4];
    bool land[4];  // interior land cell of the row (masked members)
    // raw rows in flight, indexed by row & 1
    float rq[NL][2], rh[NL][2];
};

__device__ __forceinline__ float shfl_e(float v) { return __shfl_down_sync(0xffffffffu, v, 1); }
__device__ __forceinline__ float shfl_w(float v) { return __shfl_up_sync(0xffffffffu, v, 1); }

// Issue the loads of row r (q of the stage and psi_hat, all layers / modes) into raw slot S.
template <int NL, int S>
__device__ __forceinline__ void fetch(Win<NL>& w, const float* __restrict__ qb, const float* __restrict__ hb,
                                      int64_t lstride, int r, int Ny, int x, int Nx, int Px) {
    const bool ok = r >= 0 && r < Ny && x >= 0 && x < Nx;
    const int64_t o = (int64_t)r * Px + x;
#pragma unroll
    for (int l = 0; l < NL; ++l) {
        w.rq[l][S] = ok ? __ldg(qb + l * lstride + o) : 0.f;
        w.rh[l][S] = ok ? __ldg(hb + l * lstride + o) : 0.f;
    }
}

// Ingest row r from raw slot S into window slot K = r & 3: BC, psi mix, and lap q of row
// r - 1 (window slot (K + 3) & 3, needs rows r - 2 .. r).
template <int NL, int S, int K>
__device__ __forceinline__ void ingest(Win<NL>& w, const float (&cm)[NL][NL], const Coef& c, int r, int Ny, int x,
                                       int Nx, bool apply_bc, bool zero_psi_ring, const uint8_t* mask) {
    const bool ring = r == 0 || r == Ny - 1 || x == 0 || x == Nx - 1;
    const bool land = mask && r > 0 && r < Ny - 1 && x > 0 && x < Nx - 1 && mask[(int64_t)r * Nx + x] == 0;
    w.land[K] = land;
#pragma unroll
    for (int l = 0; l < NL; ++l) w.q[l][K] = ((apply_bc && ring) || land) ? 0.f : w.rq[l][S];
#pragma unroll
    for (int l = 0; l < NL; ++l) {
        float p = 0.f;
#pragma unroll
        for (int m = 0; m < NL; ++m) p = fmaf(cm[l][m], w.rh[m][S], p);
        w.p[l][K] = ((zero_psi_ring && ring) || land) ? 0.f : p;
    }
    constexpr int K1 = (K + 3) & 3, K2 = (K + 2) & 3;
    const int r1 = r - 1;
    const bool inter = r1 > 0 && r1 < Ny - 1 && x > 0 && x < Nx - 1 && !w.land[K1];
#pragma unroll
    for (int l = 0; l < NL; ++l) {
        const float q1 = w.q[l][K1];
        const float lap = (shfl_e(q1) - 2.f * q1 + shfl_w(q1)) * c.idx2 + (w.q[l][K] - 2.f * q1 + w.q[l][K2]) * c.idy2;
        w.lq[l][K1] = inter ? lap : 0.f;
    }
}

// Output row j = r - 2 (window slot J = j & 3).  Returns true if a non-finite value was made.
template <int NL, int J>
__device__ __forceinline__ bool output(const StencilArgs& a, int Ny, int Nx, Win<NL>& w, const float (&cl)[NL][NL],
                                       const Coef& c, int j, int x, bool write, float Fj, int64_t xo, int64_t co,
                                       int64_t lstride_x, int64_t lstride_c, bool step, bool need_y0) {
    constexpr int N = (J + 1) & 3, S = (J + 3) & 3;  // rows j + 1 and j - 1
    const bool ring = j == 0 || j == Ny - 1 || x == 0 || x == Nx - 1;
    const bool land = w.land[J];  // no dynamics on land
    const float wind = c.tau0 * Fj * c.invH0;
    // y0 of the row, loaded before the arithmetic that hides its latency
    float y0[NL];
#pragma unroll
    for (int l = 0; l < NL; ++l) y0[l] = (need_y0 && write) ? __ldg(a.y0 + xo + l * lstride_x) : 0.f;
    float d[NL];
#pragma unroll
    for (int l = 0; l < NL; ++l) {
        // east / west neighbours from the adjacent lanes (every lane takes part)
        const float le = shfl_e(w.lq[l][J]), lw = shfl_w(w.lq[l][J]);
        const float fE = shfl_e(w.p[l][J]), fW = shfl_w(w.p[l][J]), fN = w.p[l][N], fS = w.p[l][S];
        const float fNE = shfl_e(w.p[l][N]), fNW = shfl_w(w.p[l][N]);
        const float fSE = shfl_e(w.p[l][S]), fSW = shfl_w(w.p[l][S]);
        const float gE = shfl_e(w.q[l][J]), gW = shfl_w(w.q[l][J]), gN = w.q[l][N], gS = w.q[l][S];
        const float gNE = shfl_e(w.q[l][N]), gNW = shfl_w(w.q[l][N]);
        const float gSE = shfl_e(w.q[l][S]), gSW = shfl_w(w.q[l][S]);
        const float jpp = (fE - fW) * (gN - gS) - (fN - fS) * (gE - gW);
        const float jpx = fE * (gNE - gSE) - fW * (gNW - gSW) - fN * (gNE - gNW) + fS * (gSE - gSW);
        const float jxp = gN * (fNE - fNW) - gS * (fSE - fSW) - gE * (fNE - fSE) + gW * (fNW - fSW);
        const float Jb = (4.f * (fE - fW) + (fNE - fNW) + (fSE - fSW)) * c.b12;
        float v = -((jpp + jpx + jxp) * c.i12 + Jb);
        if (l == 0) v += wind;
        if (l == NL - 1) {
            const float P0 = w.p[l][J];
            v -= c.kappa * ((fE - 2.f * P0 + fW) * c.idx2 + (fN - 2.f * P0 + fS) * c.idy2);
        }
        const float L0 = w.lq[l][J];
        v += c.nu * L0;
        v -= c.nu4 * ((le - 2.f * L0 + lw) * c.idx2 + (w.lq[l][N] - 2.f * L0 + w.lq[l][S]) * c.idy2);
        d[l] = ring ? (l == 0 ? wind : 0.f) : (land ? 0.f : v);
    }
    bool bad = false;
#pragma unroll
    for (int l = 0; l < NL; ++l) bad |= !isfinite(d[l]);
    if (!write) return false;
    if (!step) {
#pragma unroll
        for (int l = 0; l < NL; ++l) a.dq[co + l * lstride_c] = d[l];
        return bad;
    }
    float yn[NL];
#pragma unroll
    for (int l = 0; l < NL; ++l) {
        // the ring tendency is state independent (wind only): every consistent scheme ends
        // at y0 + dt * dq there; stage inputs carry a zero ring
        yn[l] = ring ? (a.final_stage ? y0[l] + a.dt * d[l] : 0.f) : a.a * y0[l] + a.b * (w.q[l][J] + a.dt * d[l]);
        bad |= !isfinite(yn[l]);
        a.y_next[xo + l * lstride_x] = yn[l];
    }
    if (a.xa) {
#pragma unroll
        for (int m = 0; m < NL; ++m) {
            float s = 0.f;
#pragma unroll
            for (int l = 0; l < NL; ++l) s = fmaf(cl[m][l], yn[l], s);
            s = (ring || land) ? 0.f : s;
            const int64_t o = xo + m * lstride_x;
            if (a.xa_fmt == FMT_F32) {
                static_cast<float*>(a.xa)[o] = s;
            } else {
                __nv_bfloat16* p = static_cast<__nv_bfloat16*>(a.xa);
                const __nv_bfloat16 hi = __float2bfloat16_rn(s);
                p[o] = hi;
                p[a.xplane + o] = __float2bfloat16_rn(s - __bfloat162float(hi));
            }
            if (a.xq) a.xq[o] = s;
        }
    }
    return bad;
}

// One strip item: rows [jb, je) of columns x0 .. x0 + 27 of one member, all layers.
template <int NL>
__device__ __forceinline__ bool sweep(const StencilArgs& a, const MemberDev& M, const SweepItem& it, int R) {
    const int lane = threadIdx.x & 31;
    const int Ny = M.Ny, Nx = M.Nx, Px = M.Px;
    const int x = it.sx * kOut - kHalo + lane;
    const int jb = it.sy * R, je = min(jb + R, Ny);
    const bool out_lane = lane >= kHalo && lane < kLanes - kHalo && x < Nx;
    const bool step = a.dq == nullptr;
    const bool need_y0 = step && (a.a != 0.f || a.final_stage);
    const float* P = a.params + (int64_t)it.member * QG_NPARAMS;
    Coef c;
    c.nu = P[QG_P_NU];
    c.kappa = P[QG_P_KAPPA];
    c.tau0 = P[QG_P_TAU0];
    c.nu4 = P[QG_P_NU4];
    c.idx2 = M.inv_dx2;
    c.idy2 = M.inv_dy2;
    c.i12 = M.inv_12dxdy;
    c.b12 = M.beta_12dx;
    c.invH0 = M.invH0;
    float cm[NL][NL], cl[NL][NL];
#pragma unroll
    for (int l = 0; l < NL; ++l)
#pragma unroll
        for (int m = 0; m < NL; ++m) {
            cm[l][m] = M.Cm2l[l * kMaxLayers + m];
            cl[l][m] = M.Cl2m[l * kMaxLayers + m];
        }
    const bool zero_psi_ring = !M.barotropic;
    const bool apply_bc = a.apply_bc != 0;
    // member constants in registers (M is in global memory; stores through generic pointers
    // would otherwise force reloads)
    const uint8_t* mask = M.mask;
    const float* Fp = M.F;
    const int64_t off_x = M.off_x, off_c = M.off_state;
    const int64_t lsx = (int64_t)Ny * Px, lsc = (int64_t)Ny * Nx;
    const float* qb = a.qin + M.off_x;
    const float* hb = a.psi_hat + M.off_x;
    Win<NL> w;
    // rows are walked from jb - 4 (a multiple of 4: static window slots); the output of row j
    // follows the ingest of row j + 2
    const int r0 = jb - 4;
    // rows jb - 2 .. je + 1 are needed (outputs jb .. je - 1 read rows one beyond them, and the
    // biharmonic's lap(q) one more); the two rows before and any after are skipped
    bool bad = false;
    for (int rb = r0; rb <= je + 1; rb += 4) {
#define QG_SWEEP_ROW(K)                                                                                 \
        {                                                                                               \
            const int r = rb + K;                                                                       \
            if (r >= jb - 2 && r <= je + 1)                                                             \
                ingest<NL, (K) & 1, K>(w, cm, c, r, Ny, x, Nx, apply_bc, zero_psi_ring, mask);          \
            if (r + 2 <= je + 1) fetch<NL, (K) & 1>(w, qb, hb, lsx, r + 2, Ny, x, Nx, Px);              \
            const int j = r - 2;                                                                        \
            if (j >= jb && j < je) {                                                                    \
                const float Fj = Fp[j];                                                                 \
                bad |= output<NL, ((K) + 2) & 3>(a, Ny, Nx, w, cl, c, j, x, out_lane, Fj,               \
                                                 off_x + (int64_t)j * Px + x,                           \
                                                 off_c + (int64_t)j * Nx + x, lsx, lsc, step,          \
                                                 need_y0);                                              \
            }                                                                                           \
        }
        QG_SWEEP_ROW(0)
        QG_SWEEP_ROW(1)
        QG_SWEEP_ROW(2)
        QG_SWEEP_ROW(3)
#undef QG_SWEEP_ROW
    }
    return bad;
}

// One launch per layer count present (items grouped by the members' layer count), so that
// each instantiation gets the registers its windows need.
template <int NL>
__global__ void __launch_bounds__(kWarps * 32, (NL <= 3 ? 4 : 2)) k_sweep(StencilArgs a, const SweepItem* __restrict__ items, int n_items,
                                                       int R) {
    pdl_wait();
    pdl_launch_dependents();
    const int warp = blockIdx.x * kWarps + (threadIdx.x >> 5);
    const int n_warps = gridDim.x * kWarps;
    bool bad = false;
    for (int i = warp; i < n_items; i += n_warps) {
        const SweepItem it = items[i];
        bad |= sweep<NL>(a, a.members[it.member], it, R);
    }
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0 && a.flags) atomicOr(a.flags, 1);
}

using SweepKernel = void (*)(StencilArgs, const SweepItem*, int, int);
constexpr SweepKernel kSweep[kMaxLayers] = {k_sweep<1>, k_sweep<2>, k_sweep<3>, k_sweep<4>,
                                            k_sweep<5>, k_sweep<6>, k_sweep<7>, k_sweep<8>};

}  // namespace

int sweep_columns() { return kOut; }

// items[k] .. items[k] + n_items[k]: the strips of the members with k + 1 layers.
cudaError_t launch_sweep(const StencilArgs& a, const SweepItem* const* items, const int* n_items, int R,
                         const int* grid, cudaStream_t s, bool pdl) {
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < kMaxLayers && !e; ++k)
        if (n_items[k] > 0) e = launch_k(kSweep[k], grid[k], kWarps * 32, 0, s, pdl, a, items[k], n_items[k], R);
    return e;
}

int sweep_blocks_per_sm(int nl) {
    int n = 0;
    if (nl < 1 || nl > kMaxLayers ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kSweep[nl - 1], kWarps * 32, 0) != cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}

int sweep_warps_per_block() { return kWarps; }

}  // namespace qg
