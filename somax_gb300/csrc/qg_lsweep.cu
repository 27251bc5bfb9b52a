// The fused RHS stencil as a layer-per-warp column sweep, two columns per lane.
//
// A strip is 64 columns wide and R rows high: lane L holds columns x0 - 2 + 2L and the one
// after it, lanes 1..30 produce the 60 output columns x0 .. x0 + 59 and lanes 0 and 31 are
// the two-column halo the biharmonic term reaches.  The NL warps of a strip group each own
// one layer: warp l walks down the strip with its layer's q, psi (mixed from every mode of
// psi_hat as the row arrives, Cm2l) and lap(q) in four-row register windows.  A window row
// of q or psi is held three times, as the lane's two columns and as their east and west
// shifts (one shuffle each way), so that every term of the Arakawa Jacobian is a packed
// FP32x2 operation on register pairs: the arithmetic of both columns issues as one add / mul
// / fma.  Rows stream through a per-warp ring of kDepth rows in shared memory, filled by
// per-lane asynchronous copies (cp.async, zero fill outside the strip and the member) issued
// kDepth - 1 rows ahead of their use, so the loads in flight hold no registers.  In step mode
// each output row's stage update goes through shared memory (one named barrier of the group
// per row) so that warp m writes mode m of the next stage's Cl2m operand.  Stores are
// predicated rather than branched around.
//
// Per row r (arrays relative to the member, BC = zero ring of q when apply_bc):
//   ingest(r): q(r), psi_hat(r) -> q, psi of the warp's layer, their shifts, lap q(r - 1)
//   output(r - 2): Arakawa J(psi, q) + beta term, wind, drag, nu lap q, nu4 lap(lap q), then
//                  the Shu-Osher stage update and the operand (step mode) or dq (rhs mode),
//                  as the tile stencil (qg_stencil_tile.cuh) and the one-layer-per-lane sweep
//                  (qg_sweep.cu) do; the arithmetic of a cell is the same, its rounding may
//                  differ in the last bit (fused vs separate multiply-adds).
#include <cuda_bf16.h>

#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {

namespace {

constexpr int kOutL = 60;      // output columns per strip
constexpr int kMaxWarpsL = 8;  // warps per CTA
constexpr int kDepth = 6;      // rows of the per-warp ring (rows in flight + the one in use)
constexpr unsigned kFull = 0xffffffffu;

// strips per CTA for members of nl layers (nl warps each)
__host__ __device__ constexpr int lsweep_groups(int nl) { return nl >= kMaxWarpsL ? 1 : kMaxWarpsL / nl; }

using f2 = float2;
__device__ __forceinline__ f2 F2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ f2 B2(float a) { return make_float2(a, a); }
__device__ __forceinline__ f2 add2(f2 a, f2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) { return __ffma2_rn(b, B2(-1.f), a); }  // exact b * -1
__device__ __forceinline__ f2 mul2(f2 a, f2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }

// One window row of a field: the lane's two columns c and their east / west shifts
// e = (c.y, east of c.y), w = (west of c.x, c.x).
struct Row3 {
    f2 c, e, w;
};
__device__ __forceinline__ Row3 row3(f2 c) {
    Row3 r;
    r.c = c;
    r.e = make_float2(c.y, __shfl_down_sync(kFull, c.x, 1));
    r.w = make_float2(__shfl_up_sync(kFull, c.y, 1), c.x);
    return r;
}

struct CoefL {
    float nu, kappa_l, wind_l, nu4;  // kappa_l: drag of this layer (bottom only); wind_l: 1 on the top layer
    float idx2, idy2, i12, b12;
    float invH0, tau0;
};

template <int NL>
struct WinL {
    Row3 q[4], p[4];  // four-row windows indexed by row & 3
    f2 lq[4];
    unsigned land;    // bits 2K, 2K + 1: columns 0, 1 of window row K are interior land (masked members)
};

// Ring slot of one row, per lane: q of the warp's layer, psi_hat of every mode, and y0 of the
// row two above (the output row when this row is ingested).
template <int NL>
struct Slot {
    static constexpr int NF = NL + 2;
    f2 f[NF][32];
};

__device__ __forceinline__ void cp_async8(void* dst, const void* src, bool valid) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(su32(dst)), "l"(src), "r"(valid ? 8u : 0u)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Predicated global stores: both elements of a pair when `both`, else the first alone when
// `first` (the strip's last columns at an odd member width).
__device__ __forceinline__ void st_pair(float* p, f2 v, bool both, bool first) {
    asm volatile(
        "{\n .reg .pred a, b;\n setp.ne.b32 a, %3, 0;\n setp.ne.and.b32 b, %4, 0, !a;\n"
        " @a st.global.v2.f32 [%0], {%1, %2};\n @b st.global.f32 [%0], %1;\n}\n" ::"l"(p),
        "f"(v.x), "f"(v.y), "r"((int)both), "r"((int)first));
}
__device__ __forceinline__ void st_pair_bf16(__nv_bfloat16* p, __nv_bfloat162 v, bool both, bool first) {
    const uint32_t u = (uint32_t)__bfloat16_as_ushort(v.x) | ((uint32_t)__bfloat16_as_ushort(v.y) << 16);
    asm volatile(
        "{\n .reg .pred a, b;\n setp.ne.b32 a, %2, 0;\n setp.ne.and.b32 b, %3, 0, !a;\n"
        " @a st.global.b32 [%0], %1;\n @b st.global.b16 [%0], %4;\n}\n" ::"l"(p),
        "r"(u), "r"((int)both), "r"((int)first), "h"(__bfloat16_as_ushort(v.x)));
}
__device__ __forceinline__ void st_if(float* p, float v, bool c) {
    asm volatile("{\n .reg .pred a;\n setp.ne.b32 a, %2, 0;\n @a st.global.f32 [%0], %1;\n}\n" ::"l"(p), "f"(v),
                 "r"((int)c));
}

// Per-lane column facts, constant over a strip.
struct Cols {
    int x;              // first column of the lane (even)
    bool xin;           // first column inside the member
    bool in1;           // second column inside the member
    bool ring0, ring1;  // column on the ring (x == 0 or Nx - 1)
    bool int0, int1;    // column strictly inside (ring excluded)
    bool w0, w1;        // output columns of the strip inside the member
};

// Row-walk constants of a strip.
struct Walk {
    const float* qb;  // q of the stage, layer l
    const float* hb;  // psi_hat, mode 0
    const float* yb;  // y0, layer l
    int lsx, Px, Ny, rhi, y_lo, y_hi;  // rows y_lo <= j < y_hi bring y0
};

// Issue the copies of row r into ring slot `sl` (and y0 of row r - 2 when that is an output
// row needing it) and close the copy group of the row.  Rows past the strip's last and
// outside the member, and columns outside the member, copy zeros and read nothing (the source
// is then the row base, always valid).
template <int NL>
__device__ __forceinline__ void fetch(Slot<NL>* sl, int lane, const Walk& k, const Cols& cc, int r) {
    const bool ok = cc.xin && r <= k.rhi && r >= 0 && r < k.Ny;
    const int o = ok ? r * k.Px + cc.x : 0;  // x even and Px a multiple of 32: 8-byte aligned
    cp_async8(&sl->f[0][lane], k.qb + o, ok);
#pragma unroll
    for (int m = 0; m < NL; ++m) cp_async8(&sl->f[1 + m][lane], k.hb + m * k.lsx + o, ok);
    const bool oy = cc.xin && r - 2 >= k.y_lo && r - 2 < k.y_hi;
    cp_async8(&sl->f[1 + NL][lane], k.yb + (oy ? (r - 2) * k.Px + cc.x : 0), oy);
    cp_async_commit();
}

// Ingest row r from its ring slot into window slot K = r & 3: BC, psi mix, shifts, and lap q
// of row r - 1 (window slot (K + 3) & 3, needs rows r - 2 .. r).
template <int NL, bool MASKED, int K>
__device__ __forceinline__ void ingest(WinL<NL>& w, const Slot<NL>* sl, int lane, const float (&cm)[NL],
                                       const CoefL& c, int r, int Ny, int Nx, const Cols& cc, bool apply_bc,
                                       bool zero_psi_ring, const uint8_t* mask) {
    const bool rowring = r == 0 || r == Ny - 1;
    const bool ring0 = rowring || cc.ring0, ring1 = rowring || cc.ring1;
    bool land0 = false, land1 = false;
    if constexpr (MASKED) {
        const bool rin = r > 0 && r < Ny - 1;
        const uint8_t* mr = mask + r * Nx + cc.x;
        land0 = rin && cc.int0 && mr[0] == 0;
        land1 = rin && cc.int1 && mr[1] == 0;
        w.land = (w.land & ~(3u << (2 * K))) | ((land0 ? 1u : 0u) << (2 * K)) | ((land1 ? 2u : 0u) << (2 * K));
    }
    f2 q = sl->f[0][lane];
    if ((apply_bc && ring0) || land0) q.x = 0.f;
    if ((apply_bc && ring1) || land1 || !cc.in1) q.y = 0.f;
    f2 p = mul2(B2(cm[0]), sl->f[1][lane]);
#pragma unroll
    for (int m = 1; m < NL; ++m) p = fma2(B2(cm[m]), sl->f[1 + m][lane], p);
    if ((zero_psi_ring && ring0) || land0) p.x = 0.f;
    if ((zero_psi_ring && ring1) || land1 || !cc.in1) p.y = 0.f;
    w.q[K] = row3(q);
    w.p[K] = row3(p);
    constexpr int K1 = (K + 3) & 3, K2 = (K + 2) & 3;
    const int r1 = r - 1;
    const Row3& q1 = w.q[K1];
    const f2 m2 = B2(-2.f);
    const f2 hx = fma2(m2, q1.c, add2(q1.e, q1.w));
    const f2 hy = fma2(m2, q1.c, add2(w.q[K].c, w.q[K2].c));
    const f2 lap = fma2(hx, B2(c.idx2), mul2(hy, B2(c.idy2)));
    const bool rin1 = r1 > 0 && r1 < Ny - 1;
    bool in0 = rin1 && cc.int0, in1 = rin1 && cc.int1;
    if constexpr (MASKED) {
        in0 = in0 && !((w.land >> (2 * K1)) & 1u);
        in1 = in1 && !((w.land >> (2 * K1)) & 2u);
    }
    w.lq[K1] = F2(in0 ? lap.x : 0.f, in1 ? lap.y : 0.f);
}

// Tendency of output row j (window slot J) for the warp's layer (both columns).
template <int NL, int J>
__device__ __forceinline__ f2 tendency(const WinL<NL>& w, const CoefL& c, float wind) {
    constexpr int N = (J + 1) & 3, S = (J + 3) & 3;  // rows j + 1 and j - 1
    const Row3 &PJ = w.p[J], &PN = w.p[N], &PS = w.p[S];
    const Row3 &QJ = w.q[J], &QN = w.q[N], &QS = w.q[S];
    const f2 fE = PJ.e, fW = PJ.w, fN = PN.c, fS = PS.c;
    const f2 fNE = PN.e, fNW = PN.w, fSE = PS.e, fSW = PS.w;
    const f2 gE = QJ.e, gW = QJ.w, gN = QN.c, gS = QS.c;
    const f2 gNE = QN.e, gNW = QN.w, gSE = QS.e, gSW = QS.w;
    const f2 dfx = sub2(fE, fW), dfy = sub2(fN, fS), dgx = sub2(gE, gW), dgy = sub2(gN, gS);
    const f2 jpp = sub2(mul2(dfx, dgy), mul2(dfy, dgx));
    const f2 jpx = add2(sub2(mul2(fE, sub2(gNE, gSE)), mul2(fW, sub2(gNW, gSW))),
                        sub2(mul2(fS, sub2(gSE, gSW)), mul2(fN, sub2(gNE, gNW))));
    const f2 fNd = sub2(fNE, fNW), fSd = sub2(fSE, fSW);
    const f2 jxp = add2(sub2(mul2(gN, fNd), mul2(gS, fSd)), sub2(mul2(gW, sub2(fNW, fSW)), mul2(gE, sub2(fNE, fSE))));
    const f2 Jb = mul2(fma2(B2(4.f), dfx, add2(fNd, fSd)), B2(c.b12));
    // v = -(J i12 + Jb) + wind (top layer) - kappa lap psi (bottom layer) + nu lap q - nu4 lap lap q
    f2 v = fma2(add2(add2(jpp, jpx), jxp), B2(-c.i12), fma2(Jb, B2(-1.f), B2(wind * c.wind_l)));
    const f2 m2 = B2(-2.f);
    const f2 pJ = PJ.c;
    const f2 lp = fma2(fma2(m2, pJ, add2(fE, fW)), B2(c.idx2), mul2(fma2(m2, pJ, add2(fN, fS)), B2(c.idy2)));
    v = fma2(B2(-c.kappa_l), lp, v);
    const f2 L0 = w.lq[J];
    const Row3 L = row3(L0);
    v = fma2(B2(c.nu), L0, v);
    const f2 bl = fma2(fma2(m2, L0, add2(L.e, L.w)), B2(c.idx2), mul2(fma2(m2, L0, add2(w.lq[N], w.lq[S])), B2(c.idy2)));
    return fma2(B2(-c.nu4), bl, v);
}

__device__ __forceinline__ void named_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// What an output row needs of its strip beyond the window.
struct RowCtx {
    const float* Fp;  // wind profile of the member
    float* yn;        // y_next, layer l (x-row)
    float* dq;        // dq, layer l (caller packing)
    void* xa;         // operand, mode l (x-row)
    float* xq;        // FP32 operand copy, mode l (x-row), or null
    int Ny, Nx, Px, l, lane, bar_id;
    bool step, need_y0, mix;
};

// Output row j (window slot J): tendency, then dq (rhs mode) or the stage update and, with
// the group, the operand (step mode).  Returns true if a non-finite value was written.
template <int NL, bool MASKED, int J>
__device__ __forceinline__ bool output(const StencilArgs& a, const WinL<NL>& w, const Slot<NL>* sl, const CoefL& c,
                                       const Cols& cc, const RowCtx& x, const float (&cl)[NL], f2* xbuf, int j) {
    const bool rowring = j == 0 || j == x.Ny - 1;
    const bool ring0 = rowring || cc.ring0, ring1 = rowring || cc.ring1;
    bool land0 = false, land1 = false;
    if constexpr (MASKED) {
        land0 = (w.land >> (2 * J)) & 1u;
        land1 = (w.land >> (2 * J)) & 2u;
    }
    const float wind = c.tau0 * x.Fp[j] * c.invH0;
    const int xo = j * x.Px + cc.x;
    const f2 v = tendency<NL, J>(w, c, wind);
    const float wr = wind * c.wind_l;
    const f2 d = F2(ring0 ? wr : (land0 ? 0.f : v.x), ring1 ? wr : (land1 ? 0.f : v.y));
    if (!x.step) {
        float* o = x.dq + (j * x.Nx + cc.x);  // caller packing: no pair alignment
        st_if(o, d.x, cc.w0);
        st_if(o + 1, d.y, cc.w1);
        return (cc.w0 && !isfinite(d.x)) || (cc.w1 && !isfinite(d.y));
    }
    const f2 y0 = x.need_y0 ? sl->f[1 + NL][x.lane] : B2(0.f);  // copied with row j + 2
    // the ring tendency is state independent (wind only): every consistent scheme ends at
    // y0 + dt * dq there; stage inputs carry a zero ring
    const f2 upd = fma2(B2(a.a), y0, mul2(B2(a.b), fma2(B2(a.dt), d, w.q[J].c)));
    const f2 rg = a.final_stage ? fma2(B2(a.dt), d, y0) : B2(0.f);
    const f2 yn = F2(ring0 ? rg.x : upd.x, ring1 ? rg.y : upd.y);
    const bool bad = (cc.w0 && !isfinite(yn.x)) || (cc.w1 && !isfinite(yn.y));
    st_pair(x.yn + xo, yn, cc.w1, cc.w0);
    if (!x.mix) return bad;
    // mode l of the operand from every layer's update: exchange through shared memory
    // (double-buffered by row parity, so one barrier per row suffices)
    f2* xb = xbuf + (j & 1) * NL * 32;
    xb[x.l * 32 + x.lane] = yn;
    named_sync(x.bar_id, NL * 32);
    f2 s = mul2(B2(cl[0]), xb[x.lane]);
#pragma unroll
    for (int k = 1; k < NL; ++k) s = fma2(B2(cl[k]), xb[k * 32 + x.lane], s);
    if (ring0 || land0) s.x = 0.f;
    if (ring1 || land1) s.y = 0.f;
    if (a.xa_fmt == FMT_F32) {
        st_pair(static_cast<float*>(x.xa) + xo, s, cc.w1, cc.w0);
    } else {
        __nv_bfloat16* p = static_cast<__nv_bfloat16*>(x.xa) + xo;
        const __nv_bfloat162 hi = __floats2bfloat162_rn(s.x, s.y);
        const f2 hf = __bfloat1622float2(hi);
        st_pair_bf16(p, hi, cc.w1, cc.w0);
        st_pair_bf16(p + a.xplane, __floats2bfloat162_rn(s.x - hf.x, s.y - hf.y), cc.w1, cc.w0);
    }
    if (x.xq) st_pair(x.xq + xo, s, cc.w1, cc.w0);
    return bad;
}

// One strip item: rows [jb, je) of columns x0 .. x0 + 59 of one member, layer l of the warp.
// xbuf: the group's exchange buffer, [2][NL][32] float2; ring: the warp's kDepth row slots.
template <int NL, bool MASKED>
__device__ __forceinline__ bool lsweep(const StencilArgs& a, const MemberDev& M, const SweepItem& it, int R, int l,
                                       int bar_id, f2* xbuf, Slot<NL>* ring) {
    const int lane = threadIdx.x & 31;
    const int Ny = M.Ny, Nx = M.Nx, Px = M.Px;
    Cols cc;
    cc.x = it.sx * kOutL - 2 + 2 * lane;
    cc.xin = cc.x >= 0 && cc.x < Nx;
    cc.in1 = cc.x + 1 >= 0 && cc.x + 1 < Nx;
    cc.ring0 = cc.x == 0 || cc.x == Nx - 1;
    cc.ring1 = cc.x + 1 == 0 || cc.x + 1 == Nx - 1;
    cc.int0 = cc.x > 0 && cc.x < Nx - 1;
    cc.int1 = cc.x + 1 > 0 && cc.x + 1 < Nx - 1;
    const bool out_lane = lane >= 1 && lane <= 30;
    cc.w0 = out_lane && cc.x < Nx;
    cc.w1 = out_lane && cc.x + 1 < Nx;
    const int jb = it.sy * R, je = min(jb + R, Ny);
    const float* P = a.params + (int64_t)it.member * QG_NPARAMS;
    CoefL c;
    c.nu = P[QG_P_NU];
    c.kappa_l = l == NL - 1 ? P[QG_P_KAPPA] : 0.f;
    c.wind_l = l == 0 ? 1.f : 0.f;
    c.tau0 = P[QG_P_TAU0];
    c.nu4 = P[QG_P_NU4];
    c.idx2 = M.inv_dx2;
    c.idy2 = M.inv_dy2;
    c.i12 = M.inv_12dxdy;
    c.b12 = M.beta_12dx;
    c.invH0 = M.invH0;
    float cm[NL], cl[NL];
#pragma unroll
    for (int m = 0; m < NL; ++m) {
        cm[m] = M.Cm2l[l * kMaxLayers + m];  // psi of layer l from the modes
        cl[m] = M.Cl2m[l * kMaxLayers + m];  // mode l of the operand from the layers
    }
    const bool zero_psi_ring = !M.barotropic;
    const bool apply_bc = a.apply_bc != 0;
    const uint8_t* mask = M.mask;
    const int lsx = Ny * Px, lsc = Ny * Nx;  // member planes hold < 2^31 elements
    const int64_t xl = M.off_x + (int64_t)l * lsx;
    RowCtx x;
    x.Fp = M.F;
    x.yn = a.y_next + xl;
    x.dq = a.dq ? a.dq + M.off_state + (int64_t)l * lsc : nullptr;
    x.xa = a.xa ? static_cast<void*>(a.xa_fmt == FMT_F32 ? static_cast<char*>(a.xa) + xl * 4
                                                          : static_cast<char*>(a.xa) + xl * 2)
                : nullptr;
    x.xq = a.xq ? a.xq + xl : nullptr;
    x.Ny = Ny;
    x.Nx = Nx;
    x.Px = Px;
    x.l = l;
    x.lane = lane;
    x.bar_id = bar_id;
    x.step = a.dq == nullptr;
    x.need_y0 = x.step && (a.a != 0.f || a.final_stage);
    x.mix = x.step && a.xa != nullptr;
    // rows jb - 2 .. je + 1 are needed (outputs jb .. je - 1 read rows one beyond them, and
    // the biharmonic's lap(q) one more); row jb - 2 + k goes to ring slot k mod kDepth, and
    // the copy group of a row also brings y0 of the row two above
    const int rlo = jb - 2, rhi = je + 1;
    Walk k;
    k.qb = a.qin + xl;
    k.hb = a.psi_hat + M.off_x;
    k.yb = x.need_y0 ? a.y0 + xl : k.qb;
    k.lsx = lsx;
    k.Px = Px;
    k.Ny = Ny;
    k.rhi = rhi;
    k.y_lo = jb;
    k.y_hi = x.need_y0 ? je : jb;
    WinL<NL> w;
    w.land = 0u;
    bool bad = false;
#pragma unroll 1
    for (int s = 0; s < kDepth; ++s) fetch<NL>(ring + s, lane, k, cc, rlo + s);
    Slot<NL>* sl = ring;
    Slot<NL>* const last = ring + (kDepth - 1);
    // rlo = jb - 2 is 2 mod 4 (jb is a multiple of 4): window slots 2, 3, 0, 1, ...; the
    // output of row j follows the ingest of row j + 2, then the ring slot is refilled
#define QG_LSWEEP_ROW(K, R_, OUT)                                                                        \
    {                                                                                                    \
        const int r = (R_);                                                                              \
        cp_async_wait<kDepth - 1>();                                                                     \
        ingest<NL, MASKED, K>(w, sl, lane, cm, c, r, Ny, Nx, cc, apply_bc, zero_psi_ring, mask);          \
        if (OUT) bad |= output<NL, MASKED, ((K) + 2) & 3>(a, w, sl, c, cc, x, cl, xbuf, r - 2);           \
        fetch<NL>(sl, lane, k, cc, r + kDepth);                                                          \
        sl = sl == last ? ring : sl + 1;                                                                 \
    }
    QG_LSWEEP_ROW(2, rlo, false)
    QG_LSWEEP_ROW(3, rlo + 1, false)
    QG_LSWEEP_ROW(0, rlo + 2, false)
    QG_LSWEEP_ROW(1, rlo + 3, false)
    for (int rb = jb + 2; rb <= rhi; rb += 4) {
        QG_LSWEEP_ROW(2, rb, true)
        if (rb + 1 <= rhi) QG_LSWEEP_ROW(3, rb + 1, true)
        if (rb + 2 <= rhi) QG_LSWEEP_ROW(0, rb + 2, true)
        if (rb + 3 <= rhi) QG_LSWEEP_ROW(1, rb + 3, true)
    }
#undef QG_LSWEEP_ROW
    cp_async_wait<0>();  // the ring is reused by the next strip
    return bad;
}

// Dynamic shared memory of a CTA: the warps' rings, then the groups' exchange buffers.
template <int NL>
__host__ __device__ constexpr size_t lsweep_smem() {
    return (size_t)lsweep_groups(NL) * NL * kDepth * sizeof(Slot<NL>) + (size_t)lsweep_groups(NL) * 2 * NL * 32 * 8;
}

// One launch per layer count present.  A CTA holds lsweep_groups(NL) strip groups of NL
// warps; group g works on items g, g + groups, ... of its CTA's share (all warps of a group
// walk the same strips, so their per-row barriers pair up).
template <int NL>
__global__ void __launch_bounds__(lsweep_groups(NL) * NL * 32)
    k_lsweep(StencilArgs a, const SweepItem* __restrict__ items, int n_items, int R) {
    constexpr int G = lsweep_groups(NL);
    extern __shared__ __align__(16) uint8_t lsmem[];
    pdl_wait();
    pdl_launch_dependents();
    const int warp = threadIdx.x >> 5;
    const int g = warp / NL, l = warp - g * NL;
    Slot<NL>* ring = reinterpret_cast<Slot<NL>*>(lsmem) + (size_t)warp * kDepth;
    f2* xbuf = reinterpret_cast<f2*>(lsmem + (size_t)G * NL * kDepth * sizeof(Slot<NL>)) + (size_t)g * 2 * NL * 32;
    bool bad = false;
    for (int i = blockIdx.x * G + g; i < n_items; i += gridDim.x * G) {
        const SweepItem it = items[i];
        const MemberDev& M = a.members[it.member];
        if (M.mask)
            bad |= lsweep<NL, true>(a, M, it, R, l, 1 + g, xbuf, ring);
        else
            bad |= lsweep<NL, false>(a, M, it, R, l, 1 + g, xbuf, ring);
    }
    if (__any_sync(kFull, bad) && (threadIdx.x & 31) == 0 && a.flags) atomicOr(a.flags, 1);
}

using LSweepKernel = void (*)(StencilArgs, const SweepItem*, int, int);
constexpr LSweepKernel kLSweep[kMaxLayers] = {k_lsweep<1>, k_lsweep<2>, k_lsweep<3>, k_lsweep<4>,
                                              k_lsweep<5>, k_lsweep<6>, k_lsweep<7>, k_lsweep<8>};
constexpr size_t kLSweepSmem[kMaxLayers] = {lsweep_smem<1>(), lsweep_smem<2>(), lsweep_smem<3>(), lsweep_smem<4>(),
                                            lsweep_smem<5>(), lsweep_smem<6>(), lsweep_smem<7>(), lsweep_smem<8>()};

// Allow each instantiation the dynamic shared memory its rings need (above the 48 KB default).
bool lsweep_init() {
    static bool ok = [] {
        for (int n = 0; n < kMaxLayers; ++n)
            if (cudaFuncSetAttribute(kLSweep[n], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kLSweepSmem[n]) !=
                cudaSuccess)
                return false;
        return true;
    }();
    return ok;
}

}  // namespace

int lsweep_columns() { return kOutL; }
int lsweep_strips_per_block(int nl) { return lsweep_groups(nl); }

int lsweep_blocks_per_sm(int nl) {
    int n = 0;
    if (nl < 1 || nl > kMaxLayers || !lsweep_init() ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kLSweep[nl - 1], lsweep_groups(nl) * nl * 32,
                                                      kLSweepSmem[nl - 1]) != cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}

// items[k] .. items[k] + n_items[k]: the strips of the members with k + 1 layers.
cudaError_t launch_lsweep(const StencilArgs& a, const SweepItem* const* items, const int* n_items, int R,
                          const int* grid, cudaStream_t s, bool pdl) {
    if (!lsweep_init()) return cudaErrorInvalidValue;
    cudaError_t e = cudaSuccess;
    for (int n = 0; n < kMaxLayers && !e; ++n)
        if (n_items[n] > 0)
            e = launch_k(kLSweep[n], grid[n], lsweep_groups(n + 1) * (n + 1) * 32, kLSweepSmem[n], s, pdl, a,
                         items[n], n_items[n], R);
    return e;
}

}  // namespace qg
