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
// / fma.
//
// Rows stream through a ring of kDepth row slots in shared memory that the group shares:
// warp l copies only its own fields of a row (q and y0 of layer l, psi_hat of mode l) with
// per-lane asynchronous copies (cp.async, zero fill outside the member) kDepth rows ahead,
// and reads every mode of psi_hat from the slot after the group's per-row barrier, a row
// ahead of its use.  The same barrier publishes the stage updates of an earlier row, from
// which warp m forms mode m of the next stage's Cl2m operand, so a row costs one barrier.
//
// Each strip class (lsweep_item_class) has its own kernel, so that each keeps the registers
// of its own path: interior strips (every column and row read strictly inside the member)
// carry no ring, member-edge or store predicates; edge strips apply the column rules as
// per-lane 0/1 multipliers and selects and the row rules as warp-uniform tests, each only
// where the strip meets that kind of edge (x, y or both); masked members add the land rules.  The ring slot, window slot and exchange parity of every row
// are compile-time constants of an eight-row unrolled walk (strip heights are multiples of
// 16, so the first ingested row is 6 mod 8).
//
// Per row r (arrays relative to the member, BC = zero ring of q when apply_bc):
//   ingest(r): q(r), psi_hat(r) -> q, psi of the warp's layer, their shifts, lap q(r - 1)
//   output(r - 2): Arakawa J(psi, q) + beta term, wind, drag, nu lap q, nu4 lap(lap q), then
//                  the Shu-Osher stage update (step mode) or dq (rhs mode), as the tile
//                  stencil (qg_stencil_tile.cuh) and the one-layer-per-lane sweep
//                  (qg_sweep.cu) do; the arithmetic of a cell is the same, its rounding may
//                  differ in the last bit (fused vs separate multiply-adds)
//   operand(r - 3): mode l of the next stage's operand from every layer's update of row r - 3
#include <cuda_bf16.h>

#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {

namespace {

constexpr int kOutL = kLSweepOut;  // output columns per strip
constexpr int kDepth = 8;      // ring rows of a group: the row in use + kDepth - 1 in flight
constexpr unsigned kFull = 0xffffffffu;

// strips per CTA (one group of nl warps): small CTAs let the register file hold as many
// groups per SM as it can
__host__ __device__ constexpr int lsweep_groups(int) { return 1; }

using f2 = float2;
__device__ __forceinline__ f2 F2(float a, float b) { return make_float2(a, b); }
__device__ __forceinline__ f2 B2(float a) { return make_float2(a, a); }
__device__ __forceinline__ f2 add2(f2 a, f2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ f2 sub2(f2 a, f2 b) { return __ffma2_rn(b, B2(-1.f), a); }  // exact b * -1
__device__ __forceinline__ f2 mul2(f2 a, f2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) { return __ffma2_rn(a, b, c); }

// Row r of a member is not strictly inside (the ring, or outside the member).
__device__ __forceinline__ bool ring_row(int r, int Ny) { return (unsigned)(r - 1) >= (unsigned)(Ny - 2); }

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
    float nu, kappa_l, nu4;  // kappa_l: drag of this layer (bottom only)
    float idx2, idy2, i12, b12;
    float wind_s;            // tau0 / H0 on the top layer, else 0
};

struct WinL {
    Row3 q[4], p[4];  // four-row windows indexed by row & 3
    f2 lq[4];
    unsigned land;    // bits 2K, 2K + 1: columns 0, 1 of window row K are interior land (masked members)
};

// Ring slot of one row, shared by the group: warp l fills q[l], h[l] (mode l) and y[l] (y0 of
// the row two above, the output row when this row is ingested).
template <int NL>
struct Slot {
    f2 q[NL][32];
    f2 h[NL][32];
    f2 y[NL][32];
};
constexpr int kXRows = 2;  // rows of the exchange buffer

// One row of the ring read into registers (a row ahead of its use): q of the warp's layer,
// every mode of psi_hat, and y0 of the row two above.
template <int NL>
struct RowIn {
    f2 q, h[NL], y;
};

__device__ __forceinline__ void cp_async8(uint32_t dst, const void* src, uint32_t bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8, %2;" ::"r"(dst), "l"(src), "r"(bytes) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void named_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
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
__device__ __forceinline__ f2 sel2(bool k0, bool k1, f2 v, f2 o) { return F2(k0 ? v.x : o.x, k1 ? v.y : o.y); }

// Everything a strip walk needs beyond the windows: geometry, per-lane column facts,
// copy sources, shared-memory addresses and outputs.
template <int NL>
struct Walk {
    int Ny, Nx, Px, jb, je, rhi, l, lane, bar_id;
    bool apply_bc, zero_psi_ring, step, need_y0, mix, final_stage;
    float a, b, dt;
    // per-lane column facts (edge strips)
    int x;                 // first column of the lane (even)
    uint32_t csz;          // copy size: 8 when the lane's first column is inside the member
    bool q0, q1;           // keep q of the column on read (inside; not a ring column under BC)
    bool i0, i1;           // column strictly inside (masked members' land tests)
    f2 pm;                 // psi multiplier: 1 inside, 0 outside and on a baroclinic member's ring
    f2 im;                 // 1 on columns strictly inside, else 0 (lap q, tendency, operand)
    bool w0, w1;           // output columns of the strip inside the member
    bool out;              // output lane (1..30)
    // copy sources: row offset of the lane's first column (row * Px + x, or 0 outside)
    const float* qb;       // q of the stage, layer l
    const float* hb;       // psi_hat, mode l
    const float* yb;       // y0, layer l
    // shared memory
    uint32_t s_own;        // shared address of slot 0's q[l][lane]
    const Slot<NL>* ring;  // the group's ring
    f2* xbuf;              // the group's exchange buffer [kXRows][NL][32]
    // outputs
    const float* F;        // wind profile of the member
    float f_lo, f_hi;      // F[jb + lane], F[jb + 32 + lane]: the strip's rows (R <= 64), shuffled out per row
    const uint8_t* mask;
    float* yn;             // y_next, layer l (x-row)
    float* dq;             // dq, layer l (caller packing)
    char* xa;              // operand, mode l (x-row)
    int xa_fmt;
    int64_t xplane;
    float* xq;             // FP32 operand copy, mode l (x-row), or null
};

// Copy row rf of the warp's fields (and y0 of row rf - 2 when that is an output row) into
// ring slot S = rf mod kDepth and close the row's copy group.  Rows past the strip's last are not copied
// (their group is empty); rows outside the member and columns outside it copy zeros and
// read nothing (the source is then the layer's base, always valid).
template <int NL, bool XEDGE, bool YEDGE, int S>
__device__ __forceinline__ void fetch(const Walk<NL>& k, int rf) {
    if (rf <= k.rhi) {
        const bool rok = !YEDGE || (rf >= 0 && rf < k.Ny);
        const uint32_t sz = XEDGE ? (rok ? k.csz : 0u) : (rok ? 8u : 0u);
        const int o = (XEDGE ? k.csz != 0u : true) && rok ? rf * k.Px + k.x : 0;
        const uint32_t slot = k.s_own + (uint32_t)(S * sizeof(Slot<NL>));
        cp_async8(slot, k.qb + o, sz);
        cp_async8(slot + NL * 256, k.hb + o, sz);
        if (k.need_y0 && rf - 2 >= k.jb) {
            const int oy = (XEDGE ? k.csz != 0u : true) ? (rf - 2) * k.Px + k.x : 0;
            cp_async8(slot + 2 * NL * 256, k.yb + oy, XEDGE ? k.csz : 8u);
        }
    }
    cp_async_commit();
}

// Ingest row r (read from the ring a row earlier) into window slot K = r & 3: BC, psi mix,
// shifts, and lap q of row r - 1 (window slot (K + 3) & 3, needs rows r - 2 .. r).
template <int NL, int S>
__device__ __forceinline__ void load_row(RowIn<NL>& v, const Walk<NL>& k) {
    const Slot<NL>& sl = k.ring[S];
    v.q = sl.q[k.l][k.lane];
#pragma unroll
    for (int m = 0; m < NL; ++m) v.h[m] = sl.h[m][k.lane];
    v.y = k.need_y0 ? sl.y[k.l][k.lane] : B2(0.f);
}

template <int NL, bool MASKED, bool XEDGE, bool YEDGE, int K>
__device__ __forceinline__ void ingest(WinL& w, const Walk<NL>& k, const RowIn<NL>& in, const float (&cm)[NL],
                                       const CoefL& c, int r) {
    f2 q = in.q;
    f2 p = mul2(B2(cm[0]), in.h[0]);
#pragma unroll
    for (int m = 1; m < NL; ++m) p = fma2(B2(cm[m]), in.h[m], p);
    if constexpr (XEDGE) {
        q = sel2(k.q0, k.q1, q, B2(0.f));  // a select: the ring of a caller's state may hold anything
        p = mul2(p, k.pm);
    }
    if constexpr (YEDGE) {
        if (ring_row(r, k.Ny)) {
            if (k.apply_bc) q = B2(0.f);
            if (k.zero_psi_ring) p = B2(0.f);
        }
    }
    if constexpr (MASKED) {
        const bool rin = r > 0 && r < k.Ny - 1;
        const uint8_t* mr = k.mask + r * k.Nx + k.x;
        const bool land0 = rin && k.i0 && mr[0] == 0;
        const bool land1 = rin && k.i1 && mr[1] == 0;
        w.land = (w.land & ~(3u << (2 * K))) | ((land0 ? 1u : 0u) << (2 * K)) | ((land1 ? 2u : 0u) << (2 * K));
        if (land0) q.x = p.x = 0.f;
        if (land1) q.y = p.y = 0.f;
    }
    w.q[K] = row3(q);
    w.p[K] = row3(p);
    constexpr int K1 = (K + 3) & 3, K2 = (K + 2) & 3;
    const Row3& q1 = w.q[K1];
    const f2 m2 = B2(-2.f);
    const f2 hx = fma2(m2, q1.c, add2(q1.e, q1.w));
    const f2 hy = fma2(m2, q1.c, add2(w.q[K].c, w.q[K2].c));
    f2 lap = fma2(hx, B2(c.idx2), mul2(hy, B2(c.idy2)));
    if constexpr (XEDGE) lap = mul2(lap, k.im);
    if constexpr (YEDGE) {
        if (ring_row(r - 1, k.Ny)) lap = B2(0.f);
    }
    if constexpr (MASKED) {
        if ((w.land >> (2 * K1)) & 1u) lap.x = 0.f;
        if ((w.land >> (2 * K1)) & 2u) lap.y = 0.f;
    }
    w.lq[K1] = lap;
}

// Tendency of output row j (window slot J) for the warp's layer (both columns), without the
// wind term.
template <int J>
__device__ __forceinline__ f2 tendency(const WinL& w, const CoefL& c) {
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
    // v = -(J i12 + Jb) - kappa lap psi (bottom layer) + nu lap q - nu4 lap lap q
    f2 v = fma2(add2(add2(jpp, jpx), jxp), B2(-c.i12), mul2(Jb, B2(-1.f)));
    const f2 m2 = B2(-2.f);
    // every warp of a group does the same work (they meet at a barrier every row): the drag
    // term with kappa = 0 above the bottom layer, the wind with tau0 = 0 below the top one
    const f2 pJ = PJ.c;
    const f2 lp = fma2(fma2(m2, pJ, add2(fE, fW)), B2(c.idx2), mul2(fma2(m2, pJ, add2(fN, fS)), B2(c.idy2)));
    v = fma2(B2(-c.kappa_l), lp, v);
    const f2 L0 = w.lq[J];
    const Row3 L = row3(L0);
    v = fma2(B2(c.nu), L0, v);
    const f2 bl = fma2(fma2(m2, L0, add2(L.e, L.w)), B2(c.idx2), mul2(fma2(m2, L0, add2(w.lq[N], w.lq[S])), B2(c.idy2)));
    return fma2(B2(-c.nu4), bl, v);
}

// Output row j (window slot J; y0 read with row j + 2): tendency, then dq (rhs mode) or
// the stage update, stored and published to the group for the operand (step mode).
// Accumulates yn * 0 (or dq * 0) into chk, which turns NaN on a non-finite value.
template <int NL, bool MASKED, bool XEDGE, bool YEDGE, int J>
__device__ __forceinline__ void output(const Walk<NL>& k, const WinL& w, const CoefL& c, f2 y0, int j, f2& chk) {
    const int jo = j - k.jb;
    const float wr = c.wind_s * __shfl_sync(kFull, jo < 32 ? k.f_lo : k.f_hi, jo & 31);
    // the wind alone on ring columns
    f2 d = XEDGE ? fma2(k.im, tendency<J>(w, c), B2(wr)) : add2(tendency<J>(w, c), B2(wr));
    bool rowring = false;
    if constexpr (YEDGE) {
        rowring = j == 0 || j == k.Ny - 1;
        if (rowring) d = B2(wr);
    }
    if constexpr (MASKED) {
        if ((w.land >> (2 * J)) & 1u) d.x = 0.f;
        if ((w.land >> (2 * J)) & 2u) d.y = 0.f;
    }
    if (!k.step) {
        float* o = k.dq + (j * k.Nx + k.x);  // caller packing: no pair alignment
        st_if(o, d.x, XEDGE ? k.w0 : k.out);
        st_if(o + 1, d.y, XEDGE ? k.w1 : k.out);
        chk = fma2(d, B2(0.f), chk);
        return;
    }
    // the ring tendency is state independent (wind only): every consistent scheme ends at
    // y0 + dt * dq there; stage inputs carry a zero ring
    f2 yn = fma2(B2(k.a), y0, mul2(B2(k.b), fma2(B2(k.dt), d, w.q[J].c)));
    if constexpr (XEDGE || YEDGE) {
        const f2 rg = k.final_stage ? fma2(B2(k.dt), d, y0) : B2(0.f);
        if constexpr (XEDGE) yn = sel2(k.i0, k.i1, yn, rg);  // columns outside are not stored
        if (rowring) yn = rg;
    }
    chk = fma2(yn, B2(0.f), chk);
    float* o = k.yn + (j * k.Px + k.x);
    if constexpr (XEDGE) {
        st_pair(o, yn, k.w1, k.w0);
    } else {
        if (k.out) *reinterpret_cast<f2*>(o) = yn;
    }
    if (k.mix) k.xbuf[((j & (kXRows - 1)) * NL + k.l) * 32 + k.lane] = yn;
}

// Mode l of the next stage's operand for row j from the group's updates (after the barrier
// that follows their publication).
template <int NL, bool MASKED, bool XEDGE, bool YEDGE>
__device__ __forceinline__ void operand(const Walk<NL>& k, const float (&cl)[NL], int j) {
    const f2* xb = k.xbuf + (j & (kXRows - 1)) * NL * 32 + k.lane;
    f2 s = mul2(B2(cl[0]), xb[0]);
#pragma unroll
    for (int m = 1; m < NL; ++m) s = fma2(B2(cl[m]), xb[m * 32], s);
    if constexpr (XEDGE) s = mul2(s, k.im);
    if constexpr (YEDGE) {
        if (j == 0 || j == k.Ny - 1) s = B2(0.f);
    }
    if constexpr (MASKED) {
        const bool rin = j > 0 && j < k.Ny - 1;
        const uint8_t* mr = k.mask + j * k.Nx + k.x;
        if (rin && k.i0 && mr[0] == 0) s.x = 0.f;
        if (rin && k.i1 && mr[1] == 0) s.y = 0.f;
    }
    const int xo = j * k.Px + k.x;
    const bool both = XEDGE ? k.w1 : k.out, first = XEDGE ? k.w0 : k.out;
    if (k.xa_fmt == FMT_F32) {
        st_pair(reinterpret_cast<float*>(k.xa) + xo, s, both, first);
    } else {
        __nv_bfloat16* p = reinterpret_cast<__nv_bfloat16*>(k.xa) + xo;
        const __nv_bfloat162 hi = __floats2bfloat162_rn(s.x, s.y);
        const f2 hf = __bfloat1622float2(hi);
        st_pair_bf16(p, hi, both, first);
        st_pair_bf16(p + k.xplane, __floats2bfloat162_rn(s.x - hf.x, s.y - hf.y), both, first);
    }
    if (k.xq) st_pair(k.xq + xo, s, both, first);
}

// One row of the walk: I = position in the eight-row block (row r = block base + I, the
// base being 6 mod 8), ring slot S = r & 7, window slot K = r & 3.
// Row r was read from its ring slot S = r & 7 into `cur` in the previous row; this row reads
// row r + 1 while it computes row r (ingest) and row r - 2 (output), and refills slot S with
// row r + 8.  I = position in the eight-row block (the walk's rows start at 6 mod 8), K = r & 3.
template <int NL, bool MASKED, bool XEDGE, bool YEDGE, int I>
__device__ __forceinline__ void walk_row(WinL& w, const Walk<NL>& k, RowIn<NL>& cur, const float (&cm)[NL],
                                         const float (&cl)[NL], const CoefL& c, int r, f2& chk) {
    constexpr int S = (6 + I) & 7, K = (6 + I) & 3;
    cp_async_wait<kDepth - 2>();  // this warp's copies of row r + 1 have landed
    // every warp's row r + 1 is in its slot, every warp has read row r's slot, and row r - 3's
    // updates are published
    named_sync(k.bar_id, NL * 32);
    if (k.mix && r - 3 >= k.jb) operand<NL, MASKED, XEDGE, YEDGE>(k, cl, r - 3);
    fetch<NL, XEDGE, YEDGE, S>(k, r + kDepth);
    ingest<NL, MASKED, XEDGE, YEDGE, K>(w, k, cur, cm, c, r);
    const f2 y0 = cur.y;
    if (r + 1 <= k.rhi) load_row<NL, (S + 1) & 7>(cur, k);
    if (r - 2 >= k.jb) output<NL, MASKED, XEDGE, YEDGE, (K + 2) & 3>(k, w, c, y0, r - 2, chk);
}

// One strip item: rows [jb, je) of columns x0 .. x0 + 59 of one member, layer l of the warp.
template <int NL, bool MASKED, bool XEDGE, bool YEDGE>
__device__ __forceinline__ f2 walk(Walk<NL>& k, const float (&cm)[NL], const float (&cl)[NL], const CoefL& c,
                                   f2 chk) {
    WinL w;
    w.land = 0u;
    const int rlo = k.jb - 2;
    // prologue: rows rlo .. rlo + kDepth - 1 into slots 6, 7, 0, ..., 5, then row rlo into
    // registers
    fetch<NL, XEDGE, YEDGE, 6>(k, rlo);
    fetch<NL, XEDGE, YEDGE, 7>(k, rlo + 1);
    fetch<NL, XEDGE, YEDGE, 0>(k, rlo + 2);
    fetch<NL, XEDGE, YEDGE, 1>(k, rlo + 3);
    fetch<NL, XEDGE, YEDGE, 2>(k, rlo + 4);
    fetch<NL, XEDGE, YEDGE, 3>(k, rlo + 5);
    fetch<NL, XEDGE, YEDGE, 4>(k, rlo + 6);
    fetch<NL, XEDGE, YEDGE, 5>(k, rlo + 7);
    cp_async_wait<kDepth - 1>();
    named_sync(k.bar_id, NL * 32);
    RowIn<NL> cur;
    load_row<NL, 6>(cur, k);
#pragma unroll 1
    for (int rb = rlo; rb <= k.rhi; rb += 8) {
        walk_row<NL, MASKED, XEDGE, YEDGE, 0>(w, k, cur, cm, cl, c, rb, chk);
        if (rb + 1 > k.rhi) break;
        walk_row<NL, MASKED, XEDGE, YEDGE, 1>(w, k, cur, cm, cl, c, rb + 1, chk);
        if (rb + 2 > k.rhi) break;
        walk_row<NL, MASKED, XEDGE, YEDGE, 2>(w, k, cur, cm, cl, c, rb + 2, chk);
        if (rb + 3 > k.rhi) break;
        walk_row<NL, MASKED, XEDGE, YEDGE, 3>(w, k, cur, cm, cl, c, rb + 3, chk);
        if (rb + 4 > k.rhi) break;
        walk_row<NL, MASKED, XEDGE, YEDGE, 4>(w, k, cur, cm, cl, c, rb + 4, chk);
        if (rb + 5 > k.rhi) break;
        walk_row<NL, MASKED, XEDGE, YEDGE, 5>(w, k, cur, cm, cl, c, rb + 5, chk);
        if (rb + 6 > k.rhi) break;
        walk_row<NL, MASKED, XEDGE, YEDGE, 6>(w, k, cur, cm, cl, c, rb + 6, chk);
        if (rb + 7 > k.rhi) break;
        walk_row<NL, MASKED, XEDGE, YEDGE, 7>(w, k, cur, cm, cl, c, rb + 7, chk);
    }
    // the last output row's operand; the barrier also frees the ring for the next strip
    cp_async_wait<0>();
    named_sync(k.bar_id, NL * 32);
    if (k.mix) operand<NL, MASKED, XEDGE, YEDGE>(k, cl, k.je - 1);
    return chk;
}

// Dynamic shared memory of a CTA: the groups' rings, then their exchange buffers.
template <int NL>
__host__ __device__ constexpr size_t lsweep_smem() {
    return (size_t)lsweep_groups(NL) * kDepth * sizeof(Slot<NL>) + (size_t)lsweep_groups(NL) * kXRows * NL * 32 * 8;
}

// One launch per (layer count, strip class) present.  A CTA holds lsweep_groups(NL) strip
// groups of NL warps; group g works on items g, g + groups, ... of its CTA's share (all warps
// of a group walk the same strips, so their per-row barriers pair up).
template <int NL, int CLS>
__global__ void __launch_bounds__(lsweep_groups(NL) * NL * 32)
    k_lsweep(StencilArgs a, const SweepItem* __restrict__ items, int n_items, int R) {
    constexpr int G = lsweep_groups(NL);
    extern __shared__ __align__(16) uint8_t lsmem[];
    pdl_wait();
    pdl_launch_dependents();
    const int warp = threadIdx.x >> 5;
    const int g = warp / NL, l = warp - g * NL;
    const int lane = threadIdx.x & 31;
    Slot<NL>* ring = reinterpret_cast<Slot<NL>*>(lsmem) + (size_t)g * kDepth;
    f2* xbuf = reinterpret_cast<f2*>(lsmem + (size_t)G * kDepth * sizeof(Slot<NL>)) + (size_t)g * kXRows * NL * 32;
    f2 chk = B2(0.f);
    bool misfiled = false;
    for (int i = blockIdx.x * G + g; i < n_items; i += gridDim.x * G) {
        const SweepItem it = items[i];
        const MemberDev& M = a.members[it.member];
        // the host files each strip under its class; a strip of another class would read
        // outside the member on the interior path: skip it and report
        if (lsweep_item_class(M.Ny, M.Nx, M.mask != nullptr, it.sx, it.sy, R) != CLS) {
            misfiled = true;
            continue;
        }
        Walk<NL> k;
        k.Ny = M.Ny;
        k.Nx = M.Nx;
        k.Px = M.Px;
        k.jb = it.sy * R;
        k.je = lsweep_band_end(k.Ny, it.sy, R);
        k.rhi = k.je + 1;  // outputs jb .. je - 1 read rows one beyond them, the biharmonic one more
        k.l = l;
        k.lane = lane;
        k.bar_id = 1 + g;
        k.apply_bc = a.apply_bc != 0;
        k.zero_psi_ring = !M.barotropic;
        k.step = a.dq == nullptr;
        k.need_y0 = k.step && (a.a != 0.f || a.final_stage);
        k.mix = k.step && a.xa != nullptr;
        k.final_stage = a.final_stage != 0;
        k.a = a.a;
        k.b = a.b;
        k.dt = a.dt;
        k.x = it.sx * kOutL - 2 + 2 * lane;
        const int x = k.x, Nx = k.Nx;
        const bool in0 = x >= 0 && x < Nx, in1 = x + 1 >= 0 && x + 1 < Nx;
        k.i0 = x > 0 && x < Nx - 1;
        k.i1 = x + 1 > 0 && x + 1 < Nx - 1;
        k.q0 = in0 && !(k.apply_bc && !k.i0);
        k.q1 = in1 && !(k.apply_bc && !k.i1);
        k.pm = F2(in0 && !(k.zero_psi_ring && !k.i0) ? 1.f : 0.f, in1 && !(k.zero_psi_ring && !k.i1) ? 1.f : 0.f);
        k.im = F2(k.i0 ? 1.f : 0.f, k.i1 ? 1.f : 0.f);
        k.out = lane >= 1 && lane <= 30;
        k.w0 = k.out && in0;
        k.w1 = k.out && in1;
        k.csz = in0 ? 8u : 0u;
        const int lsx = k.Ny * k.Px, lsc = k.Ny * k.Nx;  // member planes hold < 2^31 elements
        const int64_t xl = M.off_x + (int64_t)l * lsx;
        k.qb = a.qin + xl;
        k.hb = a.psi_hat + xl;  // mode l of psi_hat
        k.yb = k.need_y0 ? a.y0 + xl : k.qb;
        k.s_own = su32(&ring[0].q[l][lane]);
        k.ring = ring;
        k.xbuf = xbuf;
        k.F = M.F;
        k.f_lo = M.F[min(k.jb + lane, k.Ny - 1)];
        k.f_hi = M.F[min(k.jb + 32 + lane, k.Ny - 1)];
        k.mask = M.mask;
        k.yn = a.y_next + xl;
        k.dq = a.dq ? a.dq + M.off_state + (int64_t)l * lsc : nullptr;
        k.xa_fmt = a.xa_fmt;
        k.xplane = a.xplane;
        k.xa = a.xa ? static_cast<char*>(a.xa) + xl * (a.xa_fmt == FMT_F32 ? 4 : 2) : nullptr;
        k.xq = a.xq ? a.xq + xl : nullptr;
        const float* P = a.params + (int64_t)it.member * QG_NPARAMS;
        CoefL c;
        c.nu = P[QG_P_NU];
        c.kappa_l = l == NL - 1 ? P[QG_P_KAPPA] : 0.f;
        c.nu4 = P[QG_P_NU4];
        c.wind_s = l == 0 ? P[QG_P_TAU0] * M.invH0 : 0.f;
        c.idx2 = M.inv_dx2;
        c.idy2 = M.inv_dy2;
        c.i12 = M.inv_12dxdy;
        c.b12 = M.beta_12dx;
        float cm[NL], cl[NL];
#pragma unroll
        for (int m = 0; m < NL; ++m) {
            cm[m] = M.Cm2l[l * kMaxLayers + m];  // psi of layer l from the modes
            cl[m] = M.Cl2m[l * kMaxLayers + m];  // mode l of the operand from the layers
        }
        if constexpr (CLS == 0)
            chk = walk<NL, false, false, false>(k, cm, cl, c, chk);
        else if constexpr (CLS == 1)
            chk = walk<NL, false, true, true>(k, cm, cl, c, chk);
        else if constexpr (CLS == 2)
            chk = walk<NL, true, true, true>(k, cm, cl, c, chk);
        else if constexpr (CLS == 3)
            chk = walk<NL, false, true, false>(k, cm, cl, c, chk);
        else
            chk = walk<NL, false, false, true>(k, cm, cl, c, chk);
    }
    const bool bad = __any_sync(kFull, !isfinite(chk.x) || !isfinite(chk.y));
    if (a.flags && lane == 0) {
        if (bad) atomicOr(a.flags, 1);
        if (misfiled) atomicOr(a.flags, 4);
    }
}

using LSweepKernel = void (*)(StencilArgs, const SweepItem*, int, int);
#define QG_LSWEEP_ROW(n) k_lsweep<n, 0>, k_lsweep<n, 1>, k_lsweep<n, 2>, k_lsweep<n, 3>, k_lsweep<n, 4>
constexpr LSweepKernel kLSweep[kMaxLayers * kLSweepClasses] = {QG_LSWEEP_ROW(1), QG_LSWEEP_ROW(2), QG_LSWEEP_ROW(3),
                                                               QG_LSWEEP_ROW(4), QG_LSWEEP_ROW(5), QG_LSWEEP_ROW(6),
                                                               QG_LSWEEP_ROW(7), QG_LSWEEP_ROW(8)};
#undef QG_LSWEEP_ROW
constexpr size_t kLSweepSmem[kMaxLayers] = {lsweep_smem<1>(), lsweep_smem<2>(), lsweep_smem<3>(), lsweep_smem<4>(),
                                            lsweep_smem<5>(), lsweep_smem<6>(), lsweep_smem<7>(), lsweep_smem<8>()};

// Allow each instantiation the dynamic shared memory its ring needs (above the 48 KB default).
bool lsweep_init() {
    static bool ok = [] {
        for (int n = 0; n < kMaxLayers * kLSweepClasses; ++n)
            if (cudaFuncSetAttribute(kLSweep[n], cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kLSweepSmem[n / kLSweepClasses]) != cudaSuccess)
                return false;
        return true;
    }();
    return ok;
}

}  // namespace

int lsweep_columns() { return kOutL; }
int lsweep_strips_per_block(int nl) { return lsweep_groups(nl); }

int lsweep_blocks_per_sm(int nl, int cls) {
    int n = 0;
    if (nl < 1 || nl > kMaxLayers || cls < 0 || cls >= kLSweepClasses || !lsweep_init() ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, kLSweep[(nl - 1) * kLSweepClasses + cls],
                                                      lsweep_groups(nl) * nl * 32, kLSweepSmem[nl - 1]) != cudaSuccess)
        return 1;
    return n > 0 ? n : 1;
}

// items[g] .. items[g] + n_items[g]: the strips of class g % kLSweepClasses of the members
// with g / kLSweepClasses + 1 layers.  Strip heights must be multiples of 16 (the walk's
// compile-time ring slots assume the first ingested row is 6 mod 8) and at most 64 (the wind
// profile of a strip is held in two registers per lane).
cudaError_t launch_lsweep_group(const StencilArgs& a, const SweepItem* items, int n_items, int R, int grid, int g,
                                cudaStream_t s, bool pdl) {
    if (R <= 0 || R % 16 != 0 || R > 64 || g < 0 || g >= kMaxLayers * kLSweepClasses) return cudaErrorInvalidValue;
    if (!lsweep_init()) return cudaErrorInvalidValue;
    if (n_items <= 0) return cudaSuccess;
    const int n = g / kLSweepClasses;
    return launch_k(kLSweep[g], grid, lsweep_groups(n + 1) * (n + 1) * 32, kLSweepSmem[n], s, pdl, a, items, n_items,
                    R);
}

cudaError_t launch_lsweep(const StencilArgs& a, const SweepItem* const* items, const int* n_items, int R,
                          const int* grid, cudaStream_t s, bool pdl) {
    cudaError_t e = cudaSuccess;
    for (int g = 0; g < kMaxLayers * kLSweepClasses && !e; ++g)
        if (n_items[g] > 0) e = launch_lsweep_group(a, items[g], n_items[g], R, grid[g], g, s, pdl);
    return e;
}

}  // namespace qg
