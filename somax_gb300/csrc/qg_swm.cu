// Multilayer shallow-water right-hand side (MultilayerShallowWater2D.vector_field,
// somax/_src/models/swm/multilayer.py:150-200) and its constant-step integration.
//
// State layout: one packed float32 array (3, nl, Ny, Nx) = h, u, v per layer, row-major, one
// ghost ring; h at T points (cell centres), u at U points (east faces), v at V points (north
// faces).  The C-grid operators are finitevolx's, restated: each writes the interior and leaves
// the ring zero, the mass flux is first-order upwind on every face an interior cell needs.
//
// k_swm_stage: one Butcher stage of the step in one launch.  A CTA stages the stage input
// y + sum_m a_m K_m of its 32 x 8 tile and a one-cell halo in shared memory, with the
// boundary rules applied on read when asked (periodic wrap, or the wall rules: u = 0 on the
// west ring, the east wall face and the east ring; v = 0 on the south ring, the north wall face
// and the north ring; free slip and zero gradient elsewhere on the ring), forms each derived
// C-grid quantity once per point, and writes dh, du, dv of every layer (or, on the last stage,
// the next state y + sum_m b_m K_m).  Per layer k:
//   dh = -div(h u) (upwind h on the faces)
//   q  = (zeta + f) / h at X points (interior), f and h interpolated from T points
//   du = X_to_U(q) V_to_U(h_V v) - d_x P + [k = 0] tau0 wind_x / H0 + nu lap u - [bottom] kappa u
//   dv = -X_to_V(q) U_to_V(h_U u) - d_y P + nu lap v - [bottom] kappa v
//   P  = KE + sum_{l <= k} g'_l h_l, KE = (U_to_T(u^2) + V_to_T(v^2)) / 2 (interior)
// HBM sees the step's state and each earlier stage derivative once per stage and each output
// once: (s + 2) x 12 B per cell and layer for stage s (s derivatives in), 324 B for a Tsit5
// step; the halo re-reads hit L2.
//
// k_swm_combine: y = y0 + sum_s c_s k_s over the packed state (the stage inputs and the step
// update of the reparameterised model, whose stage inputs are projected before the right-hand
// side).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {
namespace {

constexpr int kSwTX = 32, kSwTY = 8;

struct SwmDev {
    int nl, Ny, Nx;
    float idx, idy, idx2, idy2;
    float invH0;
    int bc;           // QG_SWM_PERIODIC / QG_SWM_WALL
    const float* fx;  // f interpolated to the X rows: (f[j] + f[j + 1]) / 2
    const float* wx;  // wind pattern at the T rows
    const float* gp;  // g'_k per layer
};

// The field value at (j, i) after the boundary rules (or as stored when !bc).
// fld: 0 = h, 1 = u, 2 = v.
__device__ __forceinline__ float ld(const float* __restrict__ a, const SwmDev& d, int fld, int j, int i, bool bc) {
    if (bc) {
        if (d.bc == QG_SWM_PERIODIC) {
            j = j == 0 ? d.Ny - 2 : (j == d.Ny - 1 ? 1 : j);
            i = i == 0 ? d.Nx - 2 : (i == d.Nx - 1 ? 1 : i);
        } else {
            if (fld == 1 && (i == 0 || i >= d.Nx - 2)) return 0.f;
            if (fld == 2 && (j == 0 || j >= d.Ny - 2)) return 0.f;
            if (fld != 2) j = min(max(j, 1), d.Ny - 2);
            if (fld != 1) i = min(max(i, 1), d.Nx - 2);
        }
    }
    return __ldg(a + (int64_t)j * d.Nx + i);
}

// The cell whose value field fld (0 = h, 1 = u, 2 = v) takes at (j, i) under the boundary
// rules: (j, i) is moved there; false where the wall rules set the value to zero.
__device__ __forceinline__ bool src_cell(const SwmDev& d, int fld, int& j, int& i) {
    if (d.bc == QG_SWM_PERIODIC) {
        j = j == 0 ? d.Ny - 2 : (j == d.Ny - 1 ? 1 : j);
        i = i == 0 ? d.Nx - 2 : (i == d.Nx - 1 ? 1 : i);
        return true;
    }
    if (fld == 1 && (i == 0 || i >= d.Nx - 2)) return false;
    if (fld == 2 && (j == 0 || j >= d.Ny - 2)) return false;
    if (fld != 2) j = min(max(j, 1), d.Ny - 2);
    if (fld != 1) i = min(max(i, 1), d.Nx - 2);
    return true;
}

// Source of the stage-input value of field fld at (j, i) after the boundary rules (or as
// stored when !bc): its offset within the layer plane, or -1 where the wall rules set it to zero.
__device__ __forceinline__ int64_t src(const SwmDev& d, int fld, int j, int i, bool bc) {
    if (bc && !src_cell(d, fld, j, i)) return -1;
    return (int64_t)j * d.Nx + i;
}

// One Butcher stage of the shallow-water step, fused:
//   stage input  Y = y + sum_{m < ns} a_m K_m   (formed as it is loaded, boundary rules on read)
//   tendency     F = vector_field(Y)            (multilayer.py:150-200)
//   output       K_s = F, or on the last stage the next state y + sum_{m < ns} b_m K_m + b_ns F
struct StageArgs {
    const float* y;       // the step's state (3 fields x nl planes)
    const float* K;       // stage derivatives K_0 .. K_{ns-1}, one state apart
    float* out;
    const float* params;  // nu, kappa, tau0
    int* flags;
    int64_t n;            // floats of one state
    int ns;
    int last;             // 1: out = the next state
    int bc;               // boundary rules on read
    float a[kMaxButcher];
    float b[kMaxButcher];
};

constexpr int kStX = kSwTX + 2, kStY = kSwTY + 2, kStE = kStX * kStY;  // tile + one-cell halo
constexpr int kHalo = 2 * kStX + 2 * kSwTY;                              // halo points (84)

struct StageTables {
    float h[kStE], u[kStE], v[kStE];       // the stage input
    float q[kStE], uh[kStE], vh[kStE];     // PV at X points, u h at U points, v h at V points
    float ke[kStE], p[kStE];               // kinetic energy, cumulative hydrostatic pressure
};

// (r, c) in the haloed tile of halo point t < kHalo: the top row, the bottom row, then the
// west and east columns between them.
__device__ __forceinline__ void halo_rc(int t, int& r, int& c) {
    if (t < kStX) {
        r = 0;
        c = t;
    } else if (t < 2 * kStX) {
        r = kStY - 1;
        c = t - kStX;
    } else if (t < 2 * kStX + kSwTY) {
        r = t - 2 * kStX + 1;
        c = 0;
    } else {
        r = t - 2 * kStX - kSwTY + 1;
        c = kStX - 1;
    }
}

// The state and the NS stage derivatives at the source of each field at (jj, ii) of layer
// offset lo: v[f][0] = y, v[f][m + 1] = K_m.  INT: the tile and its halo lie inside rows and
// columns 1 .. N - 3, where no boundary rule applies.
template <int NS, bool INT>
__device__ __forceinline__ void load_point(const SwmDev& d, const StageArgs& a, int64_t field, int64_t lo, int jj,
                                           int ii, float (&v)[3][NS + 1]) {
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        int64_t o;
        if (INT)
            o = (int64_t)jj * d.Nx + ii;
        else
            o = (jj < 0 || jj >= d.Ny || ii < 0 || ii >= d.Nx) ? -1 : src(d, f, jj, ii, a.bc != 0);
        if (o < 0) {
#pragma unroll
            for (int m = 0; m <= NS; ++m) v[f][m] = 0.f;
            continue;
        }
        const int64_t off = f * field + lo + o;
        v[f][0] = __ldg(a.y + off);
#pragma unroll
        for (int m = 0; m < NS; ++m) v[f][m + 1] = __ldg(a.K + m * a.n + off);
    }
}

template <int NS>
__device__ __forceinline__ void store_input(StageTables& t, const StageArgs& a, int e, const float (&v)[3][NS + 1],
                                            float (&y3)[3]) {
#pragma unroll
    for (int f = 0; f < 3; ++f) {
        float acc = v[f][0];
#pragma unroll
        for (int m = 0; m < NS; ++m) acc = fmaf(a.a[m], v[f][m + 1], acc);
        y3[f] = acc;
    }
    t.h[e] = y3[0];
    t.u[e] = y3[1];
    t.v[e] = y3[2];
}

// The eight tables of one layer of stage input over a block of points (rows of S points, E
// points per table): h, u, v of the stage input, PV at the X points, u h at the U points,
// v h at the V points, the kinetic energy and the cumulative hydrostatic pressure.
struct Tab {
    float* b;
    int E, S;
    __device__ __forceinline__ float* h() const { return b; }
    __device__ __forceinline__ float* u() const { return b + E; }
    __device__ __forceinline__ float* v() const { return b + 2 * E; }
    __device__ __forceinline__ float* q() const { return b + 3 * E; }
    __device__ __forceinline__ float* uh() const { return b + 4 * E; }
    __device__ __forceinline__ float* vh() const { return b + 5 * E; }
    __device__ __forceinline__ float* ke() const { return b + 6 * E; }
    __device__ __forceinline__ float* p() const { return b + 7 * E; }
};

// PV, face mass fluxes, kinetic energy and the pressure sum at table point e (row r of
// `rows`, column c; T-cell (jj, ii)), each formed where a neighbouring cell reads it; the
// pressure adds g h to p.  INT: (jj, ii) is known to be strictly inside.
template <bool INT>
__device__ __forceinline__ void swm_derive(const Tab& t, const SwmDev& d, float g, int e, int r, int c, int rows,
                                           int jj, int ii, float& q, float& uh, float& vh, float& ke, float& p) {
    const int S = t.S;
    const float *h = t.h(), *u = t.u(), *v = t.v();
    q = 0.f, uh = 0.f, vh = 0.f, ke = 0.f;
    if (INT || (jj >= 1 && jj <= d.Ny - 2 && ii >= 1 && ii <= d.Nx - 2)) {
        if (r < rows - 1 && c < S - 1) {
            const float zeta = (v[e + 1] - v[e]) * d.idx - (u[e + S] - u[e]) * d.idy;
            const float hX = 0.25f * (h[e] + h[e + 1] + h[e + S] + h[e + S + 1]);
            q = (zeta + __ldg(d.fx + jj)) / hX;
        }
        if (c < S - 1) uh = 0.5f * (h[e] + h[e + 1]) * u[e];
        if (r < rows - 1) vh = 0.5f * (h[e] + h[e + S]) * v[e];
        if (r > 0 && c > 0) {
            const float ua = u[e], ub = u[e - 1], va = v[e], vb = v[e - S];
            ke = 0.25f * (ua * ua + ub * ub + va * va + vb * vb);
        }
    }
    p = fmaf(g, h[e], p);
    t.q()[e] = q;
    t.uh()[e] = uh;
    t.vh()[e] = vh;
    t.ke()[e] = ke;
    t.p()[e] = p;
}

// dh, du, dv of layer k at table point e of T-cell row j (in: strictly inside) from the tables
// and the point's own stage input (h0, u0, v0) and derived values (q0, uh0, vh0, ke0, p0).
__device__ __forceinline__ void swm_tend(const Tab& t, const SwmDev& d, int e, int j, bool in, bool top, bool bottom,
                                         float nu, float kappa, float tau0, float h0, float u0, float v0, float q0,
                                         float uh0, float vh0, float ke0, float p0, float& dh, float& du, float& dv) {
    const int S = t.S;
    const float *h = t.h(), *u = t.u(), *v = t.v();
    dh = 0.f;
    du = (top ? tau0 * __ldg(d.wx + j) * d.invH0 : 0.f) - (bottom ? kappa * u0 : 0.f);
    dv = bottom ? -kappa * v0 : 0.f;
    if (!in) return;
    const float uw = u[e - 1], vs = v[e - S];
    const float fe = u0 * (u0 > 0.f ? h0 : h[e + 1]);
    const float fw = uw * (uw > 0.f ? h[e - 1] : h0);
    const float gn = v0 * (v0 > 0.f ? h0 : h[e + S]);
    const float gs = vs * (vs > 0.f ? h[e - S] : h0);
    dh = -((fe - fw) * d.idx + (gn - gs) * d.idy);
    const float *q = t.q(), *uh = t.uh(), *vh = t.vh(), *ke = t.ke(), *p = t.p();
    const float qU = 0.5f * (q0 + q[e - S]);
    const float qV = 0.5f * (q0 + q[e - 1]);
    const float vhU = 0.25f * (vh0 + vh[e + 1] + vh[e - S] + vh[e - S + 1]);
    const float uhV = 0.25f * (uh0 + uh[e - 1] + uh[e + S] + uh[e + S - 1]);
    const float Pc = ke0 + p0, Pe = ke[e + 1] + p[e + 1];
    const float Pn = ke[e + S] + p[e + S];
    const float lu = (u[e + 1] - 2.f * u0 + uw) * d.idx2 + (u[e + S] - 2.f * u0 + u[e - S]) * d.idy2;
    const float lv = (v[e + 1] - 2.f * v0 + v[e - 1]) * d.idx2 + (v[e + S] - 2.f * v0 + vs) * d.idy2;
    du += qU * vhU - (Pe - Pc) * d.idx + nu * lu;
    dv += -qV * uhV - (Pn - Pc) * d.idy + nu * lv;
}

// A CTA owns a 32 x 8 tile of T-cells and walks the layers.  Per layer each thread loads its
// own cell's stage input (and threads 0 .. 83 one halo cell each) into shared memory, forms
// the derived C-grid quantities at the same points, then combines its own cell's tendencies
// from those tables.  The own cell's state and stage derivatives stay in registers for the
// last stage's next state.
template <int NS, bool LAST, bool INT>
__device__ __forceinline__ void stage_tile(StageTables& t, const SwmDev& d, const StageArgs& a) {
    const int tid = threadIdx.y * kSwTX + threadIdx.x;
    const int i0 = blockIdx.x * kSwTX - 1, j0 = blockIdx.y * kSwTY - 1;  // origin of the haloed tile
    const int i = i0 + 1 + threadIdx.x, j = j0 + 1 + threadIdx.y;
    const bool mine = INT || (i < d.Nx && j < d.Ny);
    const bool in = INT || (mine && j >= 1 && j <= d.Ny - 2 && i >= 1 && i <= d.Nx - 2);
    const int64_t plane = (int64_t)d.Ny * d.Nx, field = plane * d.nl;
    const float nu = a.params[0], kappa = a.params[1], tau0 = a.params[2];
    const int eo = (threadIdx.y + 1) * kStX + threadIdx.x + 1;  // own cell in the tables
    const bool halo = tid < kHalo;
    int hr = 0, hc = 0;
    if (halo) halo_rc(tid, hr, hc);
    const int he = hr * kStX + hc;
    const Tab tb{t.h, kStE, kStX};
    bool bad = false;
    float po = 0.f, ph = 0.f;  // cumulative pressure at the own and the halo cell
    // without stage derivatives to combine, the next layer's loads are issued before this layer's
    // arithmetic, so that their latency overlaps it
    constexpr bool kPrefetch = NS == 0;
    float vo[3][NS + 1], vh[3][NS + 1];
    if (kPrefetch) {
        if (mine) load_point<NS, INT>(d, a, field, 0, j, i, vo);
        if (halo) load_point<NS, INT>(d, a, field, 0, j0 + hr, i0 + hc, vh);
    }
    for (int k = 0; k < d.nl; ++k) {
        const int64_t lo = k * plane;
        float yo3[3], yh3[3];
        if (!kPrefetch) {
            if (mine) load_point<NS, INT>(d, a, field, lo, j, i, vo);
            if (halo) load_point<NS, INT>(d, a, field, lo, j0 + hr, i0 + hc, vh);
        }
        if (mine) store_input<NS>(t, a, eo, vo, yo3);
        if (halo) store_input<NS>(t, a, he, vh, yh3);
        __syncthreads();
        float vn[3][NS + 1], vhn[3][NS + 1];
        if (kPrefetch && k + 1 < d.nl) {
            if (mine) load_point<NS, INT>(d, a, field, lo + plane, j, i, vn);
            if (halo) load_point<NS, INT>(d, a, field, lo + plane, j0 + hr, i0 + hc, vhn);
        }
        const float g = __ldg(d.gp + k);
        float qo = 0.f, uho = 0.f, vho = 0.f, keo = 0.f, x0, x1, x2, x3;
        if (mine) swm_derive<INT>(tb, d, g, eo, threadIdx.y + 1, threadIdx.x + 1, kStY, j, i, qo, uho, vho, keo, po);
        if (halo) swm_derive<INT>(tb, d, g, he, hr, hc, kStY, j0 + hr, i0 + hc, x0, x1, x2, x3, ph);
        __syncthreads();
        if (mine) {
            float dh, du, dv;
            swm_tend(tb, d, eo, j, in, k == 0, k == d.nl - 1, nu, kappa, tau0, t.h[eo], t.u[eo], t.v[eo], t.q[eo],
                     t.uh[eo], t.vh[eo], t.ke[eo], t.p[eo], dh, du, dv);
            bad |= !isfinite(dh) || !isfinite(du) || !isfinite(dv);
            const int64_t o = lo + (int64_t)j * d.Nx + i;
            const float F[3] = {dh, du, dv};
#pragma unroll
            for (int f = 0; f < 3; ++f) {
                const int64_t off = f * field + o;
                float r = F[f];
                if (LAST) {
                    // the next state at the own cell as stored (not its boundary source)
                    float yo = vo[f][0], ko[NS > 0 ? NS : 1];
                    if (INT) {
#pragma unroll
                        for (int m = 0; m < NS; ++m) ko[m] = vo[f][m + 1];
                    } else {
                        yo = __ldg(a.y + off);
#pragma unroll
                        for (int m = 0; m < NS; ++m) ko[m] = __ldg(a.K + m * a.n + off);
                    }
                    r = fmaf(a.b[NS], r, yo);
#pragma unroll
                    for (int m = 0; m < NS; ++m) r = fmaf(a.b[m], ko[m], r);
                }
                a.out[off] = r;
            }
        }
        __syncthreads();
        if (kPrefetch && k + 1 < d.nl) {
#pragma unroll
            for (int f = 0; f < 3; ++f)
#pragma unroll
                for (int m = 0; m <= NS; ++m) {
                    vo[f][m] = vn[f][m];
                    vh[f][m] = vhn[f][m];
                }
        }
    }
    if (bad && a.flags) atomicOr(a.flags, 1);
}

template <int NS, bool LAST>
__global__ void __launch_bounds__(kSwTX * kSwTY) k_swm_stage(SwmDev d, StageArgs a) {
    __shared__ StageTables t;
    const int i0 = blockIdx.x * kSwTX - 1, j0 = blockIdx.y * kSwTY - 1;
    const bool interior = i0 >= 1 && i0 + kStX - 1 <= d.Nx - 3 && j0 >= 1 && j0 + kStY - 1 <= d.Ny - 3;
    if (interior)
        stage_tile<NS, LAST, true>(t, d, a);
    else
        stage_tile<NS, LAST, false>(t, d, a);
}

// ---- cluster-resident engine: every step of a small basin in one thread-block cluster -----
//
// The C CTAs of one cluster own bands of R rows of the padded grid (CTA c: rows c R ..
// c R + R - 1) and keep, in shared memory, their rows of the state, of the stage derivatives
// K_0 .. K_{ns-2} and of two stage-input buffers.  Per stage a CTA forms its rows' stage input,
// one cluster barrier publishes it, and each CTA builds its tables from its own rows plus one
// row above and below, read from the neighbouring CTAs' shared memory (the boundary rules
// may take a ring row's value from any CTA: distributed shared memory, mapa + ld.shared::cluster).
// The stage inputs alternate between the two buffers, so one barrier per stage orders both
// the reads of a buffer and its next overwrite.  The arithmetic per cell is the stage
// kernel's (swm_derive, swm_tend).

constexpr int kScThreads = 1024;

struct SwmClusterArgs {
    SwmDev d;
    float* state;          // packed state, in place
    const float* params;   // nu, kappa, tau0
    int* flags;
    int n_steps, ns, R;
    float a[kMaxButcher][kMaxButcher];  // dt * Butcher a
    float b[kMaxButcher];               // dt * Butcher b
};

__device__ __forceinline__ unsigned sc_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
// All threads of every CTA of the cluster; orders shared (local and remote) and global memory
// at cluster scope.
__device__ __forceinline__ void sc_sync() {
    asm volatile(
        "barrier.cluster.arrive.release.aligned;\n"
        "barrier.cluster.wait.acquire.aligned;" ::
            : "memory");
}
// floats of shared memory per CTA: state, ns - 1 derivatives, two stage inputs (3 nl R Nx
// each) and the eight tables of every layer over (R + 2) x Nx points
__host__ __device__ inline int64_t swm_cluster_floats(int nl, int R, int Nx, int ns) {
    return (int64_t)3 * nl * R * Nx * (ns + 2) + (int64_t)8 * nl * (R + 2) * Nx;
}

// The shared::cluster address of `p` (a location of this CTA's shared memory) in CTA `rank`.
__device__ __forceinline__ uint32_t sc_map(const float* p, unsigned rank) {
    uint32_t a;
    asm("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(a) : "r"(su32(p)), "r"(rank));
    return a;
}
// Reads of the stage inputs that a cluster barrier published; nothing writes them before the
// next barrier, so the loads need no ordering of their own.
__device__ __forceinline__ float sc_ld(uint32_t a) {
    float v;
    asm("ld.shared::cluster.f32 %0, [%1];" : "=f"(v) : "r"(a));
    return v;
}

// Row (in the padded grid) that field f of row j takes its values from under the boundary
// rules, or -1 where the wall rules make the whole row zero.
__device__ __forceinline__ int src_row(const SwmDev& d, int f, int j) {
    if (d.bc == QG_SWM_PERIODIC) return j == 0 ? d.Ny - 2 : (j == d.Ny - 1 ? 1 : j);
    if (f == 2) return (j == 0 || j >= d.Ny - 2) ? -1 : j;
    return min(max(j, 1), d.Ny - 2);
}
// Column of the same rule, or -1 where it is zero.
__device__ __forceinline__ int src_col(const SwmDev& d, int f, int i) {
    if (d.bc == QG_SWM_PERIODIC) return i == 0 ? d.Nx - 2 : (i == d.Nx - 1 ? 1 : i);
    if (f == 1) return (i == 0 || i >= d.Nx - 2) ? -1 : i;
    return min(max(i, 1), d.Nx - 2);
}

// A thread's walk over the points (k, r, i) of nk x nr x W (i fastest) in strides of
// kScThreads: the decomposition of its first point once, then carries instead of divisions.
struct Walk {
    int k, r, i, dr, di;
    __device__ __forceinline__ Walk(int x, int nr, int W) {
        const int kr = x / W;
        i = x - kr * W;
        k = kr / nr;
        r = kr - k * nr;
        dr = kScThreads / W;
        di = kScThreads - dr * W;
    }
    __device__ __forceinline__ void next(int nr, int W) {
        i += di;
        r += dr;
        if (i >= W) {
            i -= W;
            ++r;
        }
        while (r >= nr) {
            r -= nr;
            ++k;
        }
    }
};

// Per stage: (a) the stage input of the own rows (flat over the own-row arrays), a cluster
// barrier, (b) every layer's tables (one warp per table row, the rows above and below from the
// neighbouring CTAs), (c) the derived quantities of every layer at every table point (the
// cumulative pressure summed over the layers above), (d) the own cells' tendencies
// and the stage derivative or the next state; each phase hands out one point per thread.
// Three CTA barriers and one cluster barrier a stage.
__global__ void __launch_bounds__(kScThreads) k_swm_cluster(SwmClusterArgs a) {
    extern __shared__ __align__(16) float sm[];
    const SwmDev& d = a.d;
    const int W = d.Nx, R = a.R, nl = d.nl, ns = a.ns;
    const unsigned rank = sc_rank();
    const int j0 = (int)rank * R;                // first own row
    const int rows = max(0, min(R, d.Ny - j0));  // own rows (the last CTAs may have fewer)
    const int F = 3 * nl * R * W;                // floats of the own rows of one state
    float* Y = sm;                               // the state's own rows, [f][k][r][i]
    float* K = Y + F;                            // K_0 .. K_{ns-2}
    float* Yb = K + (ns - 1) * F;                // two stage-input buffers
    float* Tb = Yb + 2 * F;                      // tables, 8 (R + 2) W floats per layer
    const int E = (R + 2) * W, ER = rows + 2;
    const int64_t plane = (int64_t)d.Ny * W;
    const float nu = a.params[0], kappa = a.params[1], tau0 = a.params[2];
    const int tid = threadIdx.x;
    // the own rows in (rows beyond the grid, in the last CTAs, are zero and never read)
    for (int o = tid; o < F; o += kScThreads) {
        const int fk = o / (R * W), r = (o / W) % R, i = o % W;
        Y[o] = r < rows ? a.state[fk * plane + (int64_t)(j0 + r) * W + i] : 0.f;
    }
    __syncthreads();
    bool bad = false;
    int par = 0;
    for (int step = 0; step < a.n_steps; ++step) {
        for (int s = 0; s < ns; ++s, par ^= 1) {
            float* Yp = Yb + par * F;
            // (a)
            for (int o = tid; o < F; o += kScThreads) {
                float acc = Y[o];
                for (int m = 0; m < s; ++m) acc = fmaf(a.a[s][m], K[m * F + o], acc);
                Yp[o] = acc;
            }
            sc_sync();
            // (b) table row re of layer k holds grid row j0 - 1 + re
            Walk wb(tid, ER, W);
            for (int x = tid; x < nl * ER * W; x += kScThreads, wb.next(ER, W)) {
                const int k = wb.k, re = wb.r, i = wb.i, j = j0 - 1 + re;
                float* tk = Tb + k * 8 * E + re * W + i;  // h; u and v E and 2 E further
#pragma unroll
                for (int f = 0; f < 3; ++f) {
                    const int jj = (j >= 0 && j < d.Ny) ? src_row(d, f, j) : -1;
                    const int ii = src_col(d, f, i);
                    float v = 0.f;
                    if (jj >= 0 && ii >= 0) {
                        const unsigned owner =
                            (jj >= j0 && jj < j0 + rows) ? rank : (jj == j0 - 1 ? rank - 1 : (unsigned)(jj / R));
                        const float* ptr = Yp + ((f * nl + k) * R + (jj - (int)owner * R)) * W + ii;
                        v = owner == rank ? *ptr : sc_ld(sc_map(ptr, owner));
                    }
                    tk[f * E] = v;
                }
            }
            __syncthreads();
            // (c) one layer-point per thread; the pressure of layer k sums g'_l h_l over l < k first
            Walk wc(tid, ER, W);
            for (int x = tid; x < nl * ER * W; x += kScThreads, wc.next(ER, W)) {
                const int k = wc.k, re = wc.r, i = wc.i, e = re * W + i, j = j0 - 1 + re;
                float p = 0.f;
                for (int l = 0; l < k; ++l) p = fmaf(__ldg(d.gp + l), Tb[l * 8 * E + e], p);
                const Tab t{Tb + k * 8 * E, E, W};
                float q, uh, vh, ke;
                swm_derive<false>(t, d, __ldg(d.gp + k), e, re, i, ER, j, i, q, uh, vh, ke, p);
            }
            __syncthreads();
            // (d) one layer-cell per thread
            const bool last = s == ns - 1;
            Walk wd(tid, rows > 0 ? rows : 1, W);
            for (int x = tid; x < nl * rows * W; x += kScThreads, wd.next(rows, W)) {
                const int k = wd.k, r = wd.r, i = wd.i, j = j0 + r;
                {
                    const int e = (r + 1) * W + i;
                    const bool in = j >= 1 && j <= d.Ny - 2 && i >= 1 && i <= d.Nx - 2;
                    {
                        const Tab t{Tb + k * 8 * E, E, W};
                        float dh, du, dv;
                        swm_tend(t, d, e, j, in, k == 0, k == nl - 1, nu, kappa, tau0, t.h()[e], t.u()[e], t.v()[e],
                                 t.q()[e], t.uh()[e], t.vh()[e], t.ke()[e], t.p()[e], dh, du, dv);
                        bad |= !isfinite(dh) || !isfinite(du) || !isfinite(dv);
                        const float Fv[3] = {dh, du, dv};
#pragma unroll
                        for (int f = 0; f < 3; ++f) {
                            const int o = ((f * nl + k) * R + r) * W + i;
                            if (!last) {
                                K[s * F + o] = Fv[f];
                            } else {
                                float y = fmaf(a.b[s], Fv[f], Y[o]);
                                for (int m = 0; m < s; ++m) y = fmaf(a.b[m], K[m * F + o], y);
                                Y[o] = y;
                            }
                        }
                    }
                }
            }
            __syncthreads();
        }
    }
    for (int o = tid; o < F; o += kScThreads) {
        const int fk = o / (R * W), r = (o / W) % R, i = o % W;
        if (r < rows) a.state[fk * plane + (int64_t)(j0 + r) * W + i] = Y[o];
    }
    if (bad && a.flags) atomicOr(a.flags, 1);
    sc_sync();  // no CTA leaves while another may still read its stage input
}

// ---- adjoint of the right-hand side --------------------------------------------------------
//
// The transpose of vector_field's Jacobian at a stage input Y, applied to a cotangent
// gbar = (dh_bar, du_bar, dv_bar), as gathers in two passes:
//  k_swm_vjp_mid  the cotangents of the intermediate quantities at every point: PV at the X
//                 points (q_bar), the face mass fluxes of the PV flux (vh_bar at V points,
//                 uh_bar at U points), the Bernoulli potential at T points (P_bar = ke_bar, and
//                 the pressure sum's), and the upwind mass fluxes (Fx_bar on east faces, Fy_bar
//                 on north faces), each gathered from the tendencies that read it;
//  k_swm_vjp_in   the cotangent of the stage input (after the boundary rules) at every point,
//                 gathered from those and the direct terms (Laplacians, drag); the pressure sum
//                 sum_{l<=k} g'_l h_l becomes a reverse cumulative sum over the layers; and the
//                 parameter cotangents (nu, kappa, tau0) summed over the grid;
//  k_swm_bc_vjp   the transpose of the boundary rules: every ring or wall-face value that
//                 copied a source cell passes its cotangent on to it (zeroed values drop theirs).
// The upwind switch and the PV division are differentiated where they are smooth (the switch
// as a constant choice of upwind cell).

// Forward values of the right-hand side at any point of layer k of the stage input y, with
// the boundary rules on read when bc (the same expressions as the stage kernel's).
struct SwmAt {
    const SwmDev& d;
    const float* y;
    int64_t plane, field;
    bool bc;
    __device__ __forceinline__ bool inside(int a, int b) const {
        return a >= 1 && a <= d.Ny - 2 && b >= 1 && b <= d.Nx - 2;
    }
    __device__ __forceinline__ float H(int k, int a, int b) const { return ld(y + k * plane, d, 0, a, b, bc); }
    __device__ __forceinline__ float U(int k, int a, int b) const { return ld(y + field + k * plane, d, 1, a, b, bc); }
    __device__ __forceinline__ float V(int k, int a, int b) const {
        return ld(y + 2 * field + k * plane, d, 2, a, b, bc);
    }
    __device__ __forceinline__ float hX(int k, int a, int b) const {
        return 0.25f * (H(k, a, b) + H(k, a, b + 1) + H(k, a + 1, b) + H(k, a + 1, b + 1));
    }
    __device__ __forceinline__ float qX(int k, int a, int b) const {
        if (!inside(a, b)) return 0.f;
        const float zeta = (V(k, a, b + 1) - V(k, a, b)) * d.idx - (U(k, a + 1, b) - U(k, a, b)) * d.idy;
        return (zeta + __ldg(d.fx + a)) / hX(k, a, b);
    }
    __device__ __forceinline__ float uh(int k, int a, int b) const {
        return inside(a, b) ? 0.5f * (H(k, a, b) + H(k, a, b + 1)) * U(k, a, b) : 0.f;
    }
    __device__ __forceinline__ float vh(int k, int a, int b) const {
        return inside(a, b) ? 0.5f * (H(k, a, b) + H(k, a + 1, b)) * V(k, a, b) : 0.f;
    }
    // at an interior output cell (j, i)
    __device__ __forceinline__ float qU(int k, int j, int i) const { return 0.5f * (qX(k, j, i) + qX(k, j - 1, i)); }
    __device__ __forceinline__ float qV(int k, int j, int i) const { return 0.5f * (qX(k, j, i) + qX(k, j, i - 1)); }
    __device__ __forceinline__ float vhU(int k, int j, int i) const {
        return 0.25f * (vh(k, j, i) + vh(k, j, i + 1) + vh(k, j - 1, i) + vh(k, j - 1, i + 1));
    }
    __device__ __forceinline__ float uhV(int k, int j, int i) const {
        return 0.25f * (uh(k, j, i) + uh(k, j, i - 1) + uh(k, j + 1, i) + uh(k, j + 1, i - 1));
    }
};

// Mid-point cotangents: six planes per layer in `mid` ([k][0..5][Ny][Nx]: q_bar, vh_bar,
// uh_bar, P_bar, Fx_bar, Fy_bar).
__global__ void __launch_bounds__(kSwTX * kSwTY) k_swm_vjp_mid(SwmDev d, const float* __restrict__ y,
                                                                const float* __restrict__ gbar, float* __restrict__ mid,
                                                                int bc) {
    const int b = blockIdx.x * kSwTX + threadIdx.x;
    const int a = blockIdx.y * kSwTY + threadIdx.y;
    if (b >= d.Nx || a >= d.Ny) return;
    const int64_t plane = (int64_t)d.Ny * d.Nx, field = plane * d.nl;
    const SwmAt F{d, y, plane, field, bc != 0};
    const int64_t o = (int64_t)a * d.Nx + b;
    for (int k = 0; k < d.nl; ++k) {
        const float* gh = gbar + k * plane;
        const float* gu = gbar + field + k * plane;
        const float* gv = gbar + 2 * field + k * plane;
        auto G = [&](const float* g, int j, int i) { return g[(int64_t)j * d.Nx + i]; };
        float qb = 0.f, vhb = 0.f, uhb = 0.f;
        if (F.inside(a, b)) {
            // q(a, b) feeds qU of U(a, b), U(a + 1, b) and qV of V(a, b), V(a, b + 1)
            qb += 0.5f * (G(gu, a, b) * F.vhU(k, a, b) - G(gv, a, b) * F.uhV(k, a, b));
            if (F.inside(a + 1, b)) qb += 0.5f * G(gu, a + 1, b) * F.vhU(k, a + 1, b);
            if (F.inside(a, b + 1)) qb -= 0.5f * G(gv, a, b + 1) * F.uhV(k, a, b + 1);
            // vh(a, b) feeds vhU of U(a, b), U(a, b - 1), U(a + 1, b), U(a + 1, b - 1)
            const int uj[4] = {a, a, a + 1, a + 1}, ui[4] = {b, b - 1, b, b - 1};
#pragma unroll
            for (int t = 0; t < 4; ++t)
                if (F.inside(uj[t], ui[t])) vhb += 0.25f * G(gu, uj[t], ui[t]) * F.qU(k, uj[t], ui[t]);
            // uh(a, b) feeds uhV of V(a, b), V(a, b + 1), V(a - 1, b), V(a - 1, b + 1)
            const int vj[4] = {a, a, a - 1, a - 1}, vi[4] = {b, b + 1, b, b + 1};
#pragma unroll
            for (int t = 0; t < 4; ++t)
                if (F.inside(vj[t], vi[t])) uhb -= 0.25f * G(gv, vj[t], vi[t]) * F.qV(k, vj[t], vi[t]);
        }
        // P(a, b): Pc of U(a, b) and V(a, b), Pe of U(a, b - 1), Pn of V(a - 1, b)
        float Pb = 0.f;
        if (F.inside(a, b)) Pb += G(gu, a, b) * d.idx + G(gv, a, b) * d.idy;
        if (F.inside(a, b - 1)) Pb -= G(gu, a, b - 1) * d.idx;
        if (F.inside(a - 1, b)) Pb -= G(gv, a - 1, b) * d.idy;
        // the upwind mass flux through the east face of (a, b) (fe of (a, b), fw of (a, b + 1))
        // and through its north face (gn of (a, b), gs of (a + 1, b))
        float Fx = 0.f, Fy = 0.f;
        if (F.inside(a, b)) {
            Fx -= G(gh, a, b) * d.idx;
            Fy -= G(gh, a, b) * d.idy;
        }
        if (F.inside(a, b + 1)) Fx += G(gh, a, b + 1) * d.idx;
        if (F.inside(a + 1, b)) Fy += G(gh, a + 1, b) * d.idy;
        float* m = mid + (int64_t)k * 6 * plane + o;
        m[0] = qb;
        m[plane] = vhb;
        m[2 * plane] = uhb;
        m[3 * plane] = Pb;
        m[4 * plane] = Fx;
        m[5 * plane] = Fy;
    }
}

// The stage-input cotangent at (a, b) of every layer and the parameter cotangents
// (accumulated in pacc[0..2] as doubles: nu, kappa, tau0).
__global__ void __launch_bounds__(kSwTX * kSwTY) k_swm_vjp_in(SwmDev d, const float* __restrict__ y,
                                                               const float* __restrict__ gbar,
                                                               const float* __restrict__ mid,
                                                               const float* __restrict__ params, float* ybar,
                                                               double* pacc, int bc) {
    const int b = blockIdx.x * kSwTX + threadIdx.x;
    const int a = blockIdx.y * kSwTY + threadIdx.y;
    const bool mine = b < d.Nx && a < d.Ny;
    const int64_t plane = (int64_t)d.Ny * d.Nx, field = plane * d.nl;
    const float nu = params[0], kappa = params[1];
    float pnu = 0.f, pkap = 0.f, ptau = 0.f;
    if (mine) {
        const SwmAt F{d, y, plane, field, bc != 0};
        const int64_t o = (int64_t)a * d.Nx + b;
        auto M = [&](int k, int c, int j, int i) { return mid[((int64_t)k * 6 + c) * plane + (int64_t)j * d.Nx + i]; };
        float pcum = 0.f;  // sum over the layers k >= l of P_bar_k(a, b)
        for (int k = d.nl - 1; k >= 0; --k) {
            const float* gu = gbar + field + k * plane;
            const float* gv = gbar + 2 * field + k * plane;
            auto G = [&](const float* g, int j, int i) { return F.inside(j, i) ? g[(int64_t)j * d.Nx + i] : 0.f; };
            const float h0 = F.H(k, a, b), u0 = F.U(k, a, b), v0 = F.V(k, a, b);
            const bool east = b + 1 < d.Nx, west = b >= 1, north = a + 1 < d.Ny, south = a >= 1;
            pcum += M(k, 3, a, b);
            float hb = 0.f;  // the pressure sum's share g'_k sum_{k' >= k} P_bar_k' is added last
            // upwind mass fluxes: face (a, b) takes h(a, b) when u(a, b) > 0, face (a, b - 1) takes
            // h(a, b) when u(a, b - 1) <= 0 (the same in y)
            float ub = 0.f, vb = 0.f;
            if (east) {
                const float fx = M(k, 4, a, b);
                if (u0 > 0.f) hb += fx * u0;
                ub += fx * (u0 > 0.f ? h0 : F.H(k, a, b + 1));
            }
            if (west) {
                const float uw = F.U(k, a, b - 1);
                if (!(uw > 0.f)) hb += M(k, 4, a, b - 1) * uw;
            }
            if (north) {
                const float fy = M(k, 5, a, b);
                if (v0 > 0.f) hb += fy * v0;
                vb += fy * (v0 > 0.f ? h0 : F.H(k, a + 1, b));
            }
            if (south) {
                const float vs = F.V(k, a - 1, b);
                if (!(vs > 0.f)) hb += M(k, 5, a - 1, b) * vs;
            }
            // PV: q = (zeta + f) / hX at the X points (a, b), (a, b - 1), (a - 1, b), (a - 1, b - 1)
            auto zb = [&](int j, int i) {  // zeta_bar = q_bar / hX
                return F.inside(j, i) ? M(k, 0, j, i) / F.hX(k, j, i) : 0.f;
            };
            const int xj[4] = {a, a, a - 1, a - 1}, xi[4] = {b, b - 1, b, b - 1};
#pragma unroll
            for (int t = 0; t < 4; ++t)
                if (F.inside(xj[t], xi[t])) hb -= 0.25f * M(k, 0, xj[t], xi[t]) * F.qX(k, xj[t], xi[t]) / F.hX(k, xj[t], xi[t]);
            ub += (zb(a, b) - (south ? zb(a - 1, b) : 0.f)) * d.idy;
            vb += ((west ? zb(a, b - 1) : 0.f) - zb(a, b)) * d.idx;
            // face mass fluxes of the PV flux: vh(a, b), vh(a - 1, b), uh(a, b), uh(a, b - 1)
            hb += 0.5f * (M(k, 1, a, b) * v0 + (south ? M(k, 1, a - 1, b) * F.V(k, a - 1, b) : 0.f));
            hb += 0.5f * (M(k, 2, a, b) * u0 + (west ? M(k, 2, a, b - 1) * F.U(k, a, b - 1) : 0.f));
            if (north) vb += M(k, 1, a, b) * 0.5f * (h0 + F.H(k, a + 1, b));
            if (east) ub += M(k, 2, a, b) * 0.5f * (h0 + F.H(k, a, b + 1));
            // kinetic energy (interior T points): ke(a, b) and ke(a, b + 1) read u(a, b),
            // ke(a, b) and ke(a + 1, b) read v(a, b)
            const float pab = F.inside(a, b) ? M(k, 3, a, b) : 0.f;
            ub += 0.5f * u0 * (pab + (east && F.inside(a, b + 1) ? M(k, 3, a, b + 1) : 0.f));
            vb += 0.5f * v0 * (pab + (north && F.inside(a + 1, b) ? M(k, 3, a + 1, b) : 0.f));
            // Laplacians of the interior outputs (their transpose), and nu's cotangent
            const float gc = G(gu, a, b), gvc = G(gv, a, b);
            ub += nu * (((west ? G(gu, a, b - 1) : 0.f) + (east ? G(gu, a, b + 1) : 0.f) - 2.f * gc) * d.idx2 +
                        ((south ? G(gu, a - 1, b) : 0.f) + (north ? G(gu, a + 1, b) : 0.f) - 2.f * gc) * d.idy2);
            vb += nu * (((west ? G(gv, a, b - 1) : 0.f) + (east ? G(gv, a, b + 1) : 0.f) - 2.f * gvc) * d.idx2 +
                        ((south ? G(gv, a - 1, b) : 0.f) + (north ? G(gv, a + 1, b) : 0.f) - 2.f * gvc) * d.idy2);
            if (F.inside(a, b)) {
                const float lu = (F.U(k, a, b + 1) - 2.f * u0 + F.U(k, a, b - 1)) * d.idx2 +
                                 (F.U(k, a + 1, b) - 2.f * u0 + F.U(k, a - 1, b)) * d.idy2;
                const float lv = (F.V(k, a, b + 1) - 2.f * v0 + F.V(k, a, b - 1)) * d.idx2 +
                                 (F.V(k, a + 1, b) - 2.f * v0 + F.V(k, a - 1, b)) * d.idy2;
                pnu += gc * lu + gvc * lv;
            }
            // drag (bottom layer, every cell) and wind (top layer, every cell)
            const float guo = gu[o], gvo = gv[o];
            if (k == d.nl - 1) {
                ub -= kappa * guo;
                vb -= kappa * gvo;
                pkap -= guo * u0 + gvo * v0;
            }
            if (k == 0) ptau += guo * __ldg(d.wx + a) * d.invH0;
            hb += __ldg(d.gp + k) * pcum;
            ybar[k * plane + o] = hb;
            ybar[field + k * plane + o] = ub;
            ybar[2 * field + k * plane + o] = vb;
        }
    }
    // parameter cotangents: warp sums, one double atomic per warp
    for (int sh = 16; sh > 0; sh >>= 1) {
        pnu += __shfl_down_sync(0xffffffffu, pnu, sh);
        pkap += __shfl_down_sync(0xffffffffu, pkap, sh);
        ptau += __shfl_down_sync(0xffffffffu, ptau, sh);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(pacc + 0, (double)pnu);
        atomicAdd(pacc + 1, (double)pkap);
        atomicAdd(pacc + 2, (double)ptau);
    }
}

// The transpose of the boundary rules on a cotangent, in place: each value the rules take
// from another cell passes its cotangent on to that cell; values they set to zero drop it.
__global__ void k_swm_bc_vjp(SwmDev d, float* ybar) {
    const int i = blockIdx.x * kSwTX + threadIdx.x;
    const int j = blockIdx.y * kSwTY + threadIdx.y;
    if (i >= d.Nx || j >= d.Ny) return;
    const int64_t plane = (int64_t)d.Ny * d.Nx, field = plane * d.nl;
    for (int f = 0; f < 3; ++f) {
        int jj = j, ii = i;
        const bool keep = src_cell(d, f, jj, ii);
        if (keep && jj == j && ii == i) continue;
        for (int k = 0; k < d.nl; ++k) {
            float* g = ybar + f * field + k * plane;
            const float v = g[(int64_t)j * d.Nx + i];
            g[(int64_t)j * d.Nx + i] = 0.f;
            if (keep && v != 0.f) atomicAdd(g + (int64_t)jj * d.Nx + ii, v);
        }
    }
}

// y += alpha x, and y = alpha x, over n floats
__global__ void k_swm_axpy(float* y, const float* __restrict__ x, float alpha, int64_t n, int overwrite) {
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += nth)
        y[t] = overwrite ? alpha * x[t] : fmaf(alpha, x[t], y[t]);
}

__global__ void k_swm_pbar(const double* pacc, float* pbar, int accumulate) {
    if (threadIdx.x < QG_SWM_NPARAMS) pbar[threadIdx.x] = (float)pacc[threadIdx.x] + (accumulate ? pbar[threadIdx.x] : 0.f);
}

struct Combine {
    float c[kMaxButcher];
};

// y = y0 + sum_{s < ns} c_s k_s (k_s packed one state after another)
__global__ void k_swm_combine(float* y, const float* y0, const float* __restrict__ K, int64_t n, int ns, Combine c) {
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < n; t += nth) {
        float acc = y0[t];
        for (int s = 0; s < ns; ++s) acc = fmaf(c.c[s], K[s * n + t], acc);
        y[t] = acc;
    }
}

// The boundary rules written into the state in place (apply_boundary_conditions).  Every
// cell that changes takes its value from a cell the rules leave unchanged, so in place is safe.
__global__ void k_swm_bc(SwmDev d, float* y) {
    const int i = blockIdx.x * kSwTX + threadIdx.x;
    const int j = blockIdx.y * kSwTY + threadIdx.y;
    if (i >= d.Nx || j >= d.Ny) return;
    const bool ring = j == 0 || j == d.Ny - 1 || i == 0 || i == d.Nx - 1;
    const bool wall_face = d.bc == QG_SWM_WALL && (i == d.Nx - 2 || j == d.Ny - 2);
    if (!ring && !wall_face) return;
    const int64_t plane = (int64_t)d.Ny * d.Nx, field = plane * d.nl;
    const int64_t o = (int64_t)j * d.Nx + i;
    for (int f = 0; f < 3; ++f)
        for (int k = 0; k < d.nl; ++k) {
            float* a = y + f * field + k * plane;
            if (!ring && !((f == 1 && i == d.Nx - 2) || (f == 2 && j == d.Ny - 2))) continue;
            a[o] = ld(a, d, f, j, i, true);
        }
}

}  // namespace

}  // namespace qg

using namespace qg;

struct qg_swm_plan {
    qg_swm_desc desc;
    SwmDev d{};
    float* consts = nullptr;  // fx (Ny), wind (Ny)
    float* stage = nullptr;   // stage input (one state)
    float* K = nullptr;       // kMaxButcher stage derivatives
    float* params = nullptr;  // plan-owned copy of the params (graph-stable)
    float* proj = nullptr;    // projected stage input of qg_reparam_step
    void* stats_acc = nullptr;  // qg_swm_state_stats accumulators
    float* mid = nullptr;       // the VJP's mid-point cotangents (6 planes per layer)
    double* pacc = nullptr;     // the VJP's parameter cotangent sums
    // qg_swm_step_vjp replayed as a captured graph while its pointers, dt and scheme repeat
    cudaGraphExec_t vjp_exec = nullptr;
    const void* vjp_ptr[5] = {};
    double vjp_dt = 0.0;
    int vjp_scheme = -1;
    // qg_swm_segment_vjp replayed as a captured graph while its arguments repeat
    cudaGraphExec_t seg_exec = nullptr;
    const void* seg_ptr[5] = {};
    double seg_dt = 0.0;
    int seg_scheme = -1, seg_k = -1;
    int* flags = nullptr;
    int64_t n = 0;            // floats of one state
    int device = 0;
    int engine = QG_SWM_ENGINE_AUTO;
    // cluster configuration per stage count (C CTAs of R rows, dynamic shared memory; C = 0:
    // does not fit, -1: not yet probed)
    int cl_C[kMaxButcher + 1] = {-1, -1, -1, -1, -1, -1, -1};
    int cl_R[kMaxButcher + 1] = {};
    size_t cl_smem[kMaxButcher + 1] = {};
    bool cl_auto[kMaxButcher + 1] = {};  // AUTO takes the cluster engine (timed faster)
    float cl_ms[kMaxButcher + 1] = {}, st_ms[kMaxButcher + 1] = {};  // timed 32 steps, each engine
    // qg_swm_step replays captured graphs of 8 steps and of 1 step, while the state pointer,
    // dt and the scheme repeat
    cudaStream_t cap = nullptr;
    cudaGraphExec_t g8 = nullptr, g1 = nullptr;
    const float* g_state = nullptr;
    double g_dt = 0.0;
    int g_scheme = -1;
    // per-class event pairs around every launch while profiling (graphs bypassed then)
    bool profiling = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[QG_SWM_K_COUNT];
    size_t ev_used[QG_SWM_K_COUNT] = {};
};

namespace {
// launch() bracketed by a pair of events of class k on stream s while profiling
template <class F>
cudaError_t swm_timed(qg_swm_plan* p, int k, cudaStream_t s, F&& launch) {
    if (!p->profiling) return launch();
    auto& v = p->ev[k];
    if (p->ev_used[k] == v.size()) {
        cudaEvent_t a, b;
        if (cudaEventCreate(&a) != cudaSuccess) return cudaGetLastError();
        if (cudaEventCreate(&b) != cudaSuccess) {
            cudaEventDestroy(a);
            return cudaGetLastError();
        }
        v.emplace_back(a, b);
    }
    auto& pr = v[p->ev_used[k]++];
    cudaEventRecord(pr.first, s);
    const cudaError_t e = launch();
    cudaEventRecord(pr.second, s);
    return e;
}
}  // namespace

namespace {
int swm_validate(const qg_swm_desc& s) {
    if (s.nx < 2 || s.ny < 2 || s.n_layers < 1 || s.n_layers > QG_MAX_LAYERS) return QG_ERR_SHAPE;
    if (!(s.Lx > 0) || !(s.Ly > 0)) return QG_ERR_ARG;
    if (s.bc != QG_SWM_PERIODIC && s.bc != QG_SWM_WALL) return QG_ERR_ARG;
    if (s.wind_profile != QG_WIND_DOUBLEGYRE && s.wind_profile != QG_WIND_SINGLE) return QG_ERR_ARG;
    for (int k = 0; k < s.n_layers; ++k)
        if (!(s.H[k] > 0)) return QG_ERR_ARG;
    return QG_OK;
}
dim3 swm_grid(const SwmDev& d) { return dim3((d.Nx + kSwTX - 1) / kSwTX, (d.Ny + kSwTY - 1) / kSwTY); }
}  // namespace

extern "C" int qg_swm_create(const qg_swm_desc* desc, qg_swm_plan** out) {
    if (!desc || !out) return QG_ERR_NULL;
    *out = nullptr;
    const int v = swm_validate(*desc);
    if (v != QG_OK) return v;
    qg_swm_plan* p = new (std::nothrow) qg_swm_plan();
    if (!p) return QG_ERR_CUDA;
    p->desc = *desc;
    const qg_swm_desc& s = *desc;
    SwmDev& d = p->d;
    d.nl = s.n_layers;
    d.Ny = s.ny + 2;
    d.Nx = s.nx + 2;
    const double dx = s.Lx / s.nx, dy = s.Ly / s.ny;
    d.idx = (float)(1.0 / dx);
    d.idy = (float)(1.0 / dy);
    d.idx2 = (float)(1.0 / (dx * dx));
    d.idy2 = (float)(1.0 / (dy * dy));
    d.invH0 = (float)(1.0 / s.H[0]);
    d.bc = s.bc;
    p->n = (int64_t)3 * d.nl * d.Ny * d.Nx;
    // f at the X rows and the wind pattern at the T rows (f(y) = f0 + beta (y - Ly / 2),
    // y_j = j dy; tau_x = -cos(2 pi y / Ly) or -cos(pi y / Ly)), rounded once from float64
    std::vector<float> c(2 * (size_t)d.Ny + d.nl);
    for (int k = 0; k < d.nl; ++k) c[2 * (size_t)d.Ny + k] = (float)s.g_prime[k];
    const double kw = s.wind_profile == QG_WIND_SINGLE ? 1.0 : 2.0;
    for (int j = 0; j < d.Ny; ++j) {
        const double f0 = s.f0 + s.beta * (j * dy - s.Ly / 2.0), f1 = s.f0 + s.beta * ((j + 1) * dy - s.Ly / 2.0);
        c[j] = (float)(0.5 * (f0 + f1));
        c[d.Ny + j] = (float)(-std::cos(kw * M_PI * (j * dy) / s.Ly));
    }
    cudaError_t e = cudaGetDevice(&p->device);
    if (!e) e = cudaMalloc(&p->consts, c.size() * sizeof(float));
    if (!e) e = cudaMemcpy(p->consts, c.data(), c.size() * sizeof(float), cudaMemcpyHostToDevice);
    if (!e) e = cudaMalloc(&p->stage, p->n * sizeof(float));
    if (!e) e = cudaMalloc(&p->K, (size_t)kMaxButcher * p->n * sizeof(float));
    if (!e) e = cudaMalloc(&p->params, 4 * sizeof(float));
    if (!e) e = cudaMemset(p->params, 0, 4 * sizeof(float));
    if (!e) e = cudaMalloc(&p->proj, p->n * sizeof(float));
    if (!e) e = cudaMalloc(&p->stats_acc, 64);
    if (!e) e = cudaMalloc(&p->mid, (size_t)6 * d.nl * d.Ny * d.Nx * sizeof(float));
    if (!e) e = cudaMalloc(&p->pacc, 4 * sizeof(double));
    if (!e) e = cudaMalloc(&p->flags, 16);
    if (!e) e = cudaMemset(p->flags, 0, 16);
    if (!e) e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
    if (e) {
        qg_swm_destroy(p);
        return QG_ERR_CUDA;
    }
    d.fx = p->consts;
    d.wx = p->consts + d.Ny;
    d.gp = p->consts + 2 * d.Ny;
    *out = p;
    return QG_OK;
}

extern "C" void qg_swm_destroy(qg_swm_plan* p) {
    if (!p) return;
    cudaDeviceSynchronize();
    for (cudaGraphExec_t x : {p->g8, p->g1, p->vjp_exec, p->seg_exec})
        if (x) cudaGraphExecDestroy(x);
    for (auto& v : p->ev)
        for (auto& pr : v) {
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
    if (p->cap) cudaStreamDestroy(p->cap);
    for (void* a : {(void*)p->consts, (void*)p->stage, (void*)p->K, (void*)p->params, (void*)p->proj,
                    p->stats_acc, (void*)p->mid, (void*)p->pacc, (void*)p->flags})
        if (a) cudaFree(a);
    delete p;
}

extern "C" int64_t qg_swm_state_size(const qg_swm_plan* p) { return p ? p->n : -1; }

namespace {
// One fused stage launch (k_swm_stage) on stream s.
template <int NS>
void launch_ns(const qg_swm_plan* p, const StageArgs& a, cudaStream_t s) {
    if (a.last)
        k_swm_stage<NS, true><<<swm_grid(p->d), dim3(kSwTX, kSwTY), 0, s>>>(p->d, a);
    else
        k_swm_stage<NS, false><<<swm_grid(p->d), dim3(kSwTX, kSwTY), 0, s>>>(p->d, a);
}

cudaError_t launch_stage(const qg_swm_plan* p, const StageArgs& a, cudaStream_t s) {
    static_assert(kMaxButcher == 6, "one instantiation per stage count");
    switch (a.ns) {
        case 0: launch_ns<0>(p, a, s); break;
        case 1: launch_ns<1>(p, a, s); break;
        case 2: launch_ns<2>(p, a, s); break;
        case 3: launch_ns<3>(p, a, s); break;
        case 4: launch_ns<4>(p, a, s); break;
        case 5: launch_ns<5>(p, a, s); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

StageArgs stage_args(const qg_swm_plan* p, const float* y, float* out, const float* params, int bc) {
    StageArgs a{};
    a.y = y;
    a.K = p->K;
    a.out = out;
    a.params = params;
    a.flags = p->flags;
    a.n = p->n;
    a.bc = bc;
    return a;
}
}  // namespace

extern "C" int qg_swm_rhs(qg_swm_plan* p, const float* state, float* tend, const float* params, int flags,
                          void* stream) {
    if (!p || !state || !tend || !params) return QG_ERR_NULL;
    if (flags & ~QG_RHS_APPLY_BC) return QG_ERR_ARG;
    const StageArgs a = stage_args(p, state, tend, params, flags & QG_RHS_APPLY_BC);
    return launch_stage(p, a, (cudaStream_t)stream) == cudaSuccess ? QG_OK : QG_ERR_CUDA;
}

extern "C" int qg_swm_apply_bc(qg_swm_plan* p, float* state, void* stream) {
    if (!p || !state) return QG_ERR_NULL;
    k_swm_bc<<<swm_grid(p->d), dim3(kSwTX, kSwTY), 0, (cudaStream_t)stream>>>(p->d, state);
    return cudaGetLastError() == cudaSuccess ? QG_OK : QG_ERR_CUDA;
}

namespace {
// k steps of the Butcher-form stepper on stream s (params: the plan's copy).  Every stage is
// one k_swm_stage launch; the last stage of a step writes the next state into the other
// buffer of the pair (state, p->stage), so the steps alternate between them and an odd k
// ends with a copy back into state.
cudaError_t swm_steps(qg_swm_plan* p, float* state, const Tableau* tb, double dt, int k, cudaStream_t s) {
    float* buf[2] = {state, p->stage};
    for (int step = 0; step < k; ++step) {
        const float* y = buf[step & 1];
        for (int st = 0; st < tb->n; ++st) {
            const bool last = st == tb->n - 1;
            StageArgs a = stage_args(p, y, last ? buf[(step + 1) & 1] : p->K + st * p->n, p->params, 1);
            a.ns = st;
            a.last = last;
            for (int m = 0; m < st; ++m) a.a[m] = (float)(dt * tb->a[st][m]);
            if (last)
                for (int m = 0; m < tb->n; ++m) a.b[m] = (float)(dt * tb->b[m]);
            const cudaError_t e = swm_timed(p, QG_SWM_K_STAGE, s, [&] { return launch_stage(p, a, s); });
            if (e) return e;
        }
    }
    if (k & 1) return cudaMemcpyAsync(state, p->stage, p->n * sizeof(float), cudaMemcpyDeviceToDevice, s);
    return cudaSuccess;
}
}  // namespace

namespace {
// Whether a cluster of C CTAs holds the basin for a scheme of ns stages: shared memory within
// the device's opt-in limit and at least one such cluster resident.
bool swm_cluster_fits(const qg_swm_plan* p, int ns, int C, int* R_out, size_t* bytes_out) {
    int optin = 0;
    if (cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, p->device)) return false;
    const int R = (p->d.Ny + C - 1) / C;
    const size_t bytes = (size_t)swm_cluster_floats(p->d.nl, R, p->d.Nx, ns) * sizeof(float);
    if (bytes > (size_t)optin) return false;
    if (cudaFuncSetAttribute(k_swm_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes)) return false;
    if (C > 8 && cudaFuncSetAttribute(k_swm_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)) return false;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)C);
    cfg.blockDim = dim3(kScThreads);
    cfg.dynamicSmemBytes = bytes;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    int n = 0;
    if (cudaOccupancyMaxActiveClusters(&n, k_swm_cluster, &cfg) != cudaSuccess || n < 1) return false;
    *R_out = R;
    *bytes_out = bytes;
    return true;
}

cudaError_t launch_swm_cluster(qg_swm_plan* p, float* state, const Tableau* tb, double dt, int n_steps,
                               cudaStream_t s);

// Milliseconds of `run` on the plan's capture stream (one warm-up run first), or -1.
template <class F>
float swm_time(qg_swm_plan* p, F&& run) {
    cudaEvent_t a = nullptr, b = nullptr;
    float ms = -1.f;
    if (cudaEventCreate(&a) == cudaSuccess && cudaEventCreate(&b) == cudaSuccess && run() == cudaSuccess &&
        cudaEventRecord(a, p->cap) == cudaSuccess && run() == cudaSuccess &&
        cudaEventRecord(b, p->cap) == cudaSuccess && cudaEventSynchronize(b) == cudaSuccess)
        cudaEventElapsedTime(&ms, a, b);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    cudaGetLastError();
    return ms;
}

// Engine choice for a scheme of ns stages, once per ns (synchronises the device): every
// cluster size that fits (16, 8, 4, 2 CTAs) and the one-launch-per-stage engine (as 8-step
// graphs) each time 32 steps of the rest state in the plan's projection buffer; the fastest
// cluster size is kept for the cluster engine, and AUTO takes the cluster engine when it beat
// the stage engine.
void swm_tune(qg_swm_plan* p, const Tableau* tb) {
    const int ns = tb->n;
    if (p->cl_C[ns] >= 0) return;
    // the timing runs overwrite the plan's stage, derivative and projection buffers on the
    // plan's own stream: work of earlier calls still reading them on the caller's stream
    // finishes first
    cudaDeviceSynchronize();
    const bool prof = p->profiling;
    p->profiling = false;
    const qg_swm_desc& ds = p->desc;
    double Hs = 0.0;
    for (int k = 0; k < ds.n_layers; ++k) Hs += ds.H[k];
    const double dt = 0.1 * std::min(ds.Lx / ds.nx, ds.Ly / ds.ny) / std::sqrt(9.81 * Hs);
    std::vector<float> rest((size_t)p->n, 0.f);
    const size_t lay = (size_t)p->d.Ny * p->d.Nx;
    for (int k = 0; k < ds.n_layers; ++k)
        std::fill(rest.begin() + k * lay, rest.begin() + (k + 1) * lay, (float)ds.H[k]);
    float* y = p->proj;
    auto reset = [&] {
        return cudaMemcpyAsync(y, rest.data(), rest.size() * sizeof(float), cudaMemcpyHostToDevice, p->cap);
    };
    int bestC = 0, bestR = 0;
    size_t bestB = 0;
    float best = -1.f;
    for (int C = 16; C >= 2; C /= 2) {
        int R = 0;
        size_t bytes = 0;
        if (!swm_cluster_fits(p, ns, C, &R, &bytes)) continue;
        p->cl_C[ns] = C;  // read by launch_swm_cluster
        p->cl_R[ns] = R;
        p->cl_smem[ns] = bytes;
        const float ms = swm_time(p, [&] {
            const cudaError_t e = reset();
            return e ? e : launch_swm_cluster(p, y, tb, dt, 32, p->cap);
        });
        if (ms > 0.f && (best < 0.f || ms < best)) {
            best = ms;
            bestC = C;
            bestR = R;
            bestB = bytes;
        }
    }
    p->cl_C[ns] = bestC;
    p->cl_R[ns] = bestR;
    p->cl_smem[ns] = bestB;
    p->cl_ms[ns] = best;
    float st = -1.f;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t g = nullptr;
    if (cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
        const cudaError_t e1 = swm_steps(p, y, tb, dt, 8, p->cap);
        if (cudaStreamEndCapture(p->cap, &graph) == cudaSuccess && e1 == cudaSuccess && graph)
            if (cudaGraphInstantiate(&g, graph, 0) != cudaSuccess) g = nullptr;
        if (graph) cudaGraphDestroy(graph);
    }
    if (g) {
        st = swm_time(p, [&] {
            cudaError_t e = reset();
            for (int r = 0; r < 4 && !e; ++r) e = cudaGraphLaunch(g, p->cap);
            return e;
        });
        cudaGraphExecDestroy(g);
    }
    p->st_ms[ns] = st;
    p->cl_auto[ns] = bestC > 0 && (st < 0.f || best < st);
    p->profiling = prof;
    cudaGetLastError();
}

// Every step of one qg_swm_step call in one cluster launch.
cudaError_t launch_swm_cluster(qg_swm_plan* p, float* state, const Tableau* tb, double dt, int n_steps,
                               cudaStream_t s) {
    const int ns = tb->n, C = p->cl_C[ns];
    // plans of other sizes may have set the kernel's shared-memory limit since
    cudaError_t e = cudaFuncSetAttribute(k_swm_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)p->cl_smem[ns]);
    if (e) return e;
    SwmClusterArgs a{};
    a.d = p->d;
    a.state = state;
    a.params = p->params;
    a.flags = p->flags;
    a.n_steps = n_steps;
    a.ns = ns;
    a.R = p->cl_R[ns];
    for (int i = 0; i < ns; ++i) {
        for (int m = 0; m < i; ++m) a.a[i][m] = (float)(dt * tb->a[i][m]);
        a.b[i] = (float)(dt * tb->b[i]);
    }
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)C);
    cfg.blockDim = dim3(kScThreads);
    cfg.dynamicSmemBytes = p->cl_smem[ns];
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return swm_timed(p, QG_SWM_K_CLUSTER, s, [&] { return cudaLaunchKernelEx(&cfg, k_swm_cluster, a); });
}
}  // namespace

extern "C" int qg_swm_set_engine(qg_swm_plan* p, int engine) {
    if (!p) return QG_ERR_NULL;
    if (engine < QG_SWM_ENGINE_AUTO || engine > QG_SWM_ENGINE_CLUSTER) return QG_ERR_ARG;
    p->engine = engine;
    return QG_OK;
}

namespace {
// Whether qg_swm_step runs a scheme on the cluster engine (tunes the scheme first).
bool swm_use_cluster(qg_swm_plan* p, const Tableau* tb) {
    if (p->engine == QG_SWM_ENGINE_STAGES) return false;
    swm_tune(p, tb);
    return p->engine == QG_SWM_ENGINE_CLUSTER ? p->cl_C[tb->n] > 0 : p->cl_auto[tb->n];
}
}  // namespace

extern "C" int qg_swm_engine(qg_swm_plan* p, int scheme, int* cluster_ctas, float* times_ms) {
    if (!p) return -QG_ERR_NULL;
    const Tableau* tb = swm_tableau(scheme);
    if (!tb) return -QG_ERR_ARG;
    const bool cl = swm_use_cluster(p, tb);
    if (cluster_ctas) *cluster_ctas = cl ? p->cl_C[tb->n] : 0;
    if (times_ms) {
        times_ms[0] = p->cl_C[tb->n] >= 0 ? p->cl_ms[tb->n] : -1.f;
        times_ms[1] = p->cl_C[tb->n] >= 0 ? p->st_ms[tb->n] : -1.f;
    }
    return cl ? QG_SWM_ENGINE_CLUSTER : QG_SWM_ENGINE_STAGES;
}

extern "C" int qg_swm_step(qg_swm_plan* p, float* state, const float* params, double dt, int n_steps, int scheme,
                           int flags, void* stream) {
    if (!p || !state || !params) return QG_ERR_NULL;
    if (n_steps < 0 || (flags & ~QG_STEP_APPLY_BC) || !(dt == dt)) return QG_ERR_ARG;
    const Tableau* tb = swm_tableau(scheme);
    if (!tb) return QG_ERR_ARG;
    const bool cluster = swm_use_cluster(p, tb);
    if (p->engine == QG_SWM_ENGINE_CLUSTER && !cluster) return QG_ERR_UNSUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(p->params, params, 3 * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (!e && (flags & QG_STEP_APPLY_BC)) {
        k_swm_bc<<<swm_grid(p->d), dim3(kSwTX, kSwTY), 0, s>>>(p->d, state);
        e = cudaGetLastError();
    }
    if (e || n_steps == 0) return e ? QG_ERR_CUDA : QG_OK;
    if (cluster) return launch_swm_cluster(p, state, tb, dt, n_steps, s) ? QG_ERR_CUDA : QG_OK;
    if (p->g_state != state || p->g_dt != dt || p->g_scheme != scheme) {
        for (cudaGraphExec_t* x : {&p->g8, &p->g1})
            if (*x) {
                cudaGraphExecDestroy(*x);
                *x = nullptr;
            }
        p->g_state = state;
        p->g_dt = dt;
        p->g_scheme = scheme;
    }
    auto capture = [&](int k, cudaGraphExec_t* out) {
        cudaGraph_t graph = nullptr;
        cudaError_t ec = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
        if (!ec) {
            const cudaError_t e1 = swm_steps(p, state, tb, dt, k, p->cap);
            ec = cudaStreamEndCapture(p->cap, &graph);
            if (!ec) ec = e1;
        }
        if (!ec) ec = cudaGraphInstantiate(out, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (ec) *out = nullptr;
        return ec;
    };
    if (p->profiling) return swm_steps(p, state, tb, dt, n_steps, s) ? QG_ERR_CUDA : QG_OK;
    int left = n_steps;
    if (left >= 8 && !p->g8) e = capture(8, &p->g8);
    for (; left >= 8 && !e; left -= 8) e = cudaGraphLaunch(p->g8, s);
    if (!e && left > 0 && !p->g1) e = capture(1, &p->g1);
    for (; left > 0 && !e; --left) e = cudaGraphLaunch(p->g1, s);
    return e ? QG_ERR_CUDA : QG_OK;
}

extern "C" int qg_swm_set_profiling(qg_swm_plan* p, int enable) {
    if (!p) return QG_ERR_NULL;
    if (cudaDeviceSynchronize() != cudaSuccess) return QG_ERR_CUDA;
    p->profiling = enable != 0;
    for (auto& u : p->ev_used) u = 0;
    return QG_OK;
}

extern "C" int qg_swm_kernel_stats(qg_swm_plan* p, int k, double* total_ms, int64_t* launches) {
    if (!p || !total_ms || !launches) return QG_ERR_NULL;
    if (k < 0 || k >= QG_SWM_K_COUNT) return QG_ERR_ARG;
    double t = 0.0;
    for (size_t i = 0; i < p->ev_used[k]; ++i) {
        if (cudaEventSynchronize(p->ev[k][i].second) != cudaSuccess) return QG_ERR_CUDA;
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p->ev[k][i].first, p->ev[k][i].second) == cudaSuccess) t += ms;
    }
    *total_ms = t;
    *launches = (int64_t)p->ev_used[k];
    return QG_OK;
}

extern "C" int qg_reparam_step(qg_swm_plan* p, qg_plan* qp, float* state, const float* params, double dt,
                               int n_steps, int scheme, int flags, void* stream) {
    if (!p || !qp || !state || !params) return QG_ERR_NULL;
    if (n_steps < 0 || (flags & ~QG_STEP_APPLY_BC) || !(dt == dt)) return QG_ERR_ARG;
    const Tableau* tb = swm_tableau(scheme);
    if (!tb) return QG_ERR_ARG;
    if (p->desc.bc != QG_SWM_WALL) return QG_ERR_ARG;
    const int64_t lay = p->n / 3;  // floats of one field (n_layers planes)
    if (qg_plan_state_size(qp) != lay) return QG_ERR_SHAPE;
    cudaStream_t s = (cudaStream_t)stream;
    const dim3 g = swm_grid(p->d), b(kSwTX, kSwTY);
    const int cgrid = (int)std::min<int64_t>(4096, (p->n + 255) / 256);
    // apply_boundary_conditions of the reparameterised model on x: the wall rules in place,
    // then the geostrophic projection into p->proj (and back into x when copy)
    auto bc_project = [&](float* x, bool copy) -> int {
        k_swm_bc<<<g, b, 0, s>>>(p->d, x);
        if (cudaGetLastError() != cudaSuccess) return QG_ERR_CUDA;
        const int r = qg_project(qp, x, x + lay, x + 2 * lay, p->proj, p->proj + lay, p->proj + 2 * lay, nullptr, s);
        if (r != QG_OK || !copy) return r;
        return cudaMemcpyAsync(x, p->proj, p->n * sizeof(float), cudaMemcpyDeviceToDevice, s) == cudaSuccess
                   ? QG_OK
                   : QG_ERR_CUDA;
    };
    cudaError_t e = cudaMemcpyAsync(p->params, params, 3 * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (e) return QG_ERR_CUDA;
    int r = QG_OK;
    if (flags & QG_STEP_APPLY_BC) r = bc_project(state, true);
    for (int step = 0; step < n_steps && r == QG_OK; ++step) {
        for (int st = 0; st < tb->n && r == QG_OK; ++st) {
            if (st == 0) {
                e = cudaMemcpyAsync(p->stage, state, p->n * sizeof(float), cudaMemcpyDeviceToDevice, s);
            } else {
                Combine c{};
                for (int j = 0; j < st; ++j) c.c[j] = (float)(dt * tb->a[st][j]);
                k_swm_combine<<<cgrid, 256, 0, s>>>(p->stage, state, p->K, p->n, st, c);
                e = cudaGetLastError();
            }
            if (e) return QG_ERR_CUDA;
            r = bc_project(p->stage, false);
            if (r != QG_OK) break;
            if (launch_stage(p, stage_args(p, p->proj, p->K + st * p->n, p->params, 0), s)) return QG_ERR_CUDA;
        }
        if (r != QG_OK) break;
        Combine c{};
        for (int j = 0; j < tb->n; ++j) c.c[j] = (float)(dt * tb->b[j]);
        k_swm_combine<<<cgrid, 256, 0, s>>>(state, state, p->K, p->n, tb->n, c);
        if (cudaGetLastError() != cudaSuccess) return QG_ERR_CUDA;
    }
    return r;
}

namespace {
// ybar = (the transpose of vector_field's Jacobian at y, with the boundary rules on read when bc)
// applied to gbar; the parameter cotangents added to p->pacc.
cudaError_t swm_vjp(qg_swm_plan* p, const float* y, const float* params, const float* gbar, float* ybar, int bc,
                    cudaStream_t s) {
    const dim3 g = swm_grid(p->d), b(kSwTX, kSwTY);
    k_swm_vjp_mid<<<g, b, 0, s>>>(p->d, y, gbar, p->mid, bc);
    k_swm_vjp_in<<<g, b, 0, s>>>(p->d, y, gbar, p->mid, params, ybar, p->pacc, bc);
    if (bc) k_swm_bc_vjp<<<g, b, 0, s>>>(p->d, ybar);
    return cudaGetLastError();
}

const Tableau* swm_scheme(int scheme) { return swm_tableau(scheme); }
}  // namespace

extern "C" int qg_swm_rhs_vjp(qg_swm_plan* p, const float* state, const float* params, const float* tend_bar,
                              float* state_bar, float* params_bar, int flags, void* stream) {
    if (!p || !state || !params || !tend_bar || !state_bar || !params_bar) return QG_ERR_NULL;
    if (flags & ~QG_RHS_APPLY_BC) return QG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemsetAsync(p->pacc, 0, 4 * sizeof(double), s);
    if (!e) e = swm_vjp(p, state, params, tend_bar, state_bar, flags & QG_RHS_APPLY_BC, s);
    if (!e) {
        k_swm_pbar<<<1, 32, 0, s>>>(p->pacc, params_bar, 0);
        e = cudaGetLastError();
    }
    return e ? QG_ERR_CUDA : QG_OK;
}

extern "C" int qg_swm_bc_vjp(qg_swm_plan* p, float* state_bar, void* stream) {
    if (!p || !state_bar) return QG_ERR_NULL;
    k_swm_bc_vjp<<<swm_grid(p->d), dim3(kSwTX, kSwTY), 0, (cudaStream_t)stream>>>(p->d, state_bar);
    return cudaGetLastError() == cudaSuccess ? QG_OK : QG_ERR_CUDA;
}

extern "C" int64_t qg_swm_step_vjp_workspace(const qg_swm_plan* p, int scheme) {
    const Tableau* tb = swm_scheme(scheme);
    if (!p || !tb) return -1;
    return (int64_t)(3 * tb->n - 1) * p->n;
}

namespace {
// The launches of one step's adjoint on stream s (see qg_swm_step_vjp).
cudaError_t swm_step_vjp_body(qg_swm_plan* p, const float* y0, const float* params, double dt, const Tableau* tb,
                              float* y_bar, float* params_bar, float* work, cudaStream_t s, bool own_pacc = true) {
    const int ns = tb->n;
    const int64_t n = p->n;
    const int cgrid = (int)std::min<int64_t>(4096, (n + 255) / 256);
    // work: stage inputs Y_1 .. Y_{ns-1}, stage derivatives K_0 .. K_{ns-2} (contiguous), their
    // cotangents Kbar_0 .. Kbar_{ns-1}, one stage-input cotangent
    const float* Y[kMaxButcher];
    Y[0] = y0;
    for (int i = 1; i < ns; ++i) Y[i] = work + (int64_t)(i - 1) * n;
    float* K = work + (int64_t)(ns - 1) * n;
    float* Kb = work + (int64_t)(2 * ns - 2) * n;
    float* Yb = work + (int64_t)(3 * ns - 2) * n;
    cudaError_t e = cudaSuccess;
    // the step's stage inputs again: Y_s = y0 + dt sum_m a_sm K_m, K_m = F(B(Y_m))
    for (int st = 0; st + 1 < ns && !e; ++st) {
        e = launch_stage(p, stage_args(p, Y[st], K + st * n, params, 1), s);
        if (e) break;
        Combine c{};
        for (int m = 0; m <= st; ++m) c.c[m] = (float)(dt * tb->a[st + 1][m]);
        k_swm_combine<<<cgrid, 256, 0, s>>>(const_cast<float*>(Y[st + 1]), y0, K, n, st + 1, c);
        e = cudaGetLastError();
    }
    // Kbar_s = dt b_s ybar, then the stages in reverse: Ybar = F_vjp(Y_s; Kbar_s),
    // y0_bar += Ybar, Kbar_m += dt a_sm Ybar
    for (int st = 0; st < ns && !e; ++st) {
        k_swm_axpy<<<cgrid, 256, 0, s>>>(Kb + st * n, y_bar, (float)(dt * tb->b[st]), n, 1);
        e = cudaGetLastError();
    }
    if (!e && own_pacc) e = cudaMemsetAsync(p->pacc, 0, 4 * sizeof(double), s);
    for (int st = ns - 1; st >= 0 && !e; --st) {
        e = swm_vjp(p, Y[st], params, Kb + st * n, Yb, 1, s);
        if (e) break;
        k_swm_axpy<<<cgrid, 256, 0, s>>>(y_bar, Yb, 1.f, n, 0);
        for (int m = 0; m < st; ++m)
            if (tb->a[st][m] != 0.0) k_swm_axpy<<<cgrid, 256, 0, s>>>(Kb + m * n, Yb, (float)(dt * tb->a[st][m]), n, 0);
        e = cudaGetLastError();
    }
    if (!e && own_pacc) {
        k_swm_pbar<<<1, 32, 0, s>>>(p->pacc, params_bar, 0);
        e = cudaGetLastError();
    }
    return e;
}

// The adjoint of k steps from y_start on stream s: the k - 1 later states recomputed into
// work (one step each, the stage engine), then each step's adjoint in reverse, the parameter
// cotangents summed over the steps into params_bar.
cudaError_t swm_segment_vjp_body(qg_swm_plan* p, const float* y_start, const float* params, double dt,
                                 const Tableau* tb, int k, float* y_bar, float* params_bar, float* work,
                                 cudaStream_t s) {
    const int64_t n = p->n;
    float* states = work;                        // y_1 .. y_{k-1}
    float* vwork = work + (int64_t)(k - 1) * n;  // one step's adjoint workspace
    cudaError_t e = cudaSuccess;
    for (int i = 1; i < k && !e; ++i) {
        float* y = states + (int64_t)(i - 1) * n;
        e = cudaMemcpyAsync(y, i == 1 ? y_start : y - n, n * sizeof(float), cudaMemcpyDeviceToDevice, s);
        if (!e) e = swm_steps(p, y, tb, dt, 1, s);
    }
    if (!e) e = cudaMemsetAsync(p->pacc, 0, 4 * sizeof(double), s);
    for (int i = k - 1; i >= 0 && !e; --i) {
        const float* y = i == 0 ? y_start : states + (int64_t)(i - 1) * n;
        e = swm_step_vjp_body(p, y, params, dt, tb, y_bar, params_bar, vwork, s, false);
    }
    if (!e) {
        k_swm_pbar<<<1, 32, 0, s>>>(p->pacc, params_bar, 0);
        e = cudaGetLastError();
    }
    return e;
}
}  // namespace

extern "C" int qg_swm_step_vjp(qg_swm_plan* p, const float* y0, const float* params, double dt, int scheme,
                               float* y_bar, float* params_bar, float* work, void* stream) {
    if (!p || !y0 || !params || !y_bar || !params_bar || !work) return QG_ERR_NULL;
    const Tableau* tb = swm_scheme(scheme);
    if (!tb || !(dt == dt)) return QG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (p->profiling) return swm_step_vjp_body(p, y0, params, dt, tb, y_bar, params_bar, work, s) ? QG_ERR_CUDA : QG_OK;
    // ~9 launches per stage: captured once per set of arguments and replayed while they repeat
    // (callers that stage every step's state and cotangent in the same buffers replay it every step)
    const void* ptr[5] = {y0, params, y_bar, params_bar, work};
    bool same = p->vjp_exec && p->vjp_dt == dt && p->vjp_scheme == scheme;
    for (int k = 0; k < 5 && same; ++k) same = p->vjp_ptr[k] == ptr[k];
    cudaError_t e = cudaSuccess;
    if (!same) {
        if (p->vjp_exec) {
            cudaGraphExecDestroy(p->vjp_exec);
            p->vjp_exec = nullptr;
        }
        cudaGraph_t graph = nullptr;
        e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
        if (!e) {
            const cudaError_t e1 = swm_step_vjp_body(p, y0, params, dt, tb, y_bar, params_bar, work, p->cap);
            e = cudaStreamEndCapture(p->cap, &graph);
            if (!e) e = e1;
        }
        if (!e) e = cudaGraphInstantiate(&p->vjp_exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e) {
            p->vjp_exec = nullptr;
            return QG_ERR_CUDA;
        }
        for (int k = 0; k < 5; ++k) p->vjp_ptr[k] = ptr[k];
        p->vjp_dt = dt;
        p->vjp_scheme = scheme;
    }
    return cudaGraphLaunch(p->vjp_exec, s) == cudaSuccess ? QG_OK : QG_ERR_CUDA;
}

extern "C" int64_t qg_swm_segment_vjp_workspace(const qg_swm_plan* p, int scheme, int k) {
    const Tableau* tb = swm_scheme(scheme);
    if (!p || !tb || k < 1) return -1;
    return (int64_t)(k - 1 + 3 * tb->n - 1) * p->n;
}

extern "C" int qg_swm_segment_vjp(qg_swm_plan* p, const float* y_start, const float* params, double dt, int k,
                                  int scheme, float* y_bar, float* params_bar, float* work, void* stream) {
    if (!p || !y_start || !params || !y_bar || !params_bar || !work) return QG_ERR_NULL;
    const Tableau* tb = swm_scheme(scheme);
    if (!tb || !(dt == dt) || k < 1) return QG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (p->profiling)
        return swm_segment_vjp_body(p, y_start, params, dt, tb, k, y_bar, params_bar, work, s) ? QG_ERR_CUDA : QG_OK;
    const void* ptr[5] = {y_start, params, y_bar, params_bar, work};
    bool same = p->seg_exec && p->seg_dt == dt && p->seg_scheme == scheme && p->seg_k == k;
    for (int i = 0; i < 5 && same; ++i) same = p->seg_ptr[i] == ptr[i];
    if (!same) {
        if (p->seg_exec) {
            cudaGraphExecDestroy(p->seg_exec);
            p->seg_exec = nullptr;
        }
        cudaGraph_t graph = nullptr;
        cudaError_t e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
        if (!e) {
            const cudaError_t e1 = swm_segment_vjp_body(p, y_start, params, dt, tb, k, y_bar, params_bar, work, p->cap);
            e = cudaStreamEndCapture(p->cap, &graph);
            if (!e) e = e1;
        }
        if (!e) e = cudaGraphInstantiate(&p->seg_exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e) {
            p->seg_exec = nullptr;
            return QG_ERR_CUDA;
        }
        for (int i = 0; i < 5; ++i) p->seg_ptr[i] = ptr[i];
        p->seg_dt = dt;
        p->seg_scheme = scheme;
        p->seg_k = k;
    }
    return cudaGraphLaunch(p->seg_exec, s) == cudaSuccess ? QG_OK : QG_ERR_CUDA;
}

extern "C" int qg_swm_state_stats(qg_swm_plan* p, const float* x, int64_t n, double* stats, void* stream) {
    if (!p || !x || !stats) return QG_ERR_NULL;
    if (n < 1) return QG_ERR_ARG;
    int dev = 0, n_sm = 0;
    if (cudaGetDevice(&dev) || cudaDeviceGetAttribute(&n_sm, cudaDevAttrMultiProcessorCount, dev)) return QG_ERR_CUDA;
    const int grid = std::max(1, std::min(n_sm * 4, (int)((n / 4 + 255) / 256)));
    return launch_state_stats(x, n, p->stats_acc, stats, grid, (cudaStream_t)stream) == cudaSuccess ? QG_OK
                                                                                                   : QG_ERR_CUDA;
}

namespace {
// t = P(B(y)) (the reparameterised model's boundary conditions) through scratch t (a copy of
// y with the wall rules) into out
int reparam_bc_project(qg_swm_plan* p, qg_plan* qp, const float* y, float* t, float* out, cudaStream_t s) {
    const int64_t lay = p->n / 3;
    if (cudaMemcpyAsync(t, y, p->n * sizeof(float), cudaMemcpyDeviceToDevice, s)) return QG_ERR_CUDA;
    k_swm_bc<<<swm_grid(p->d), dim3(kSwTX, kSwTY), 0, s>>>(p->d, t);
    if (cudaGetLastError() != cudaSuccess) return QG_ERR_CUDA;
    return qg_project(qp, t, t + lay, t + 2 * lay, out, out + lay, out + 2 * lay, nullptr, s);
}

// out = B^T P^T g (the transpose of reparam_bc_project)
int reparam_bc_project_vjp(qg_swm_plan* p, qg_plan* qp, const float* g, float* out, cudaStream_t s) {
    const int64_t lay = p->n / 3;
    const int r = qg_project_vjp(qp, g, g + lay, g + 2 * lay, out, out + lay, out + 2 * lay, s);
    if (r != QG_OK) return r;
    k_swm_bc_vjp<<<swm_grid(p->d), dim3(kSwTX, kSwTY), 0, s>>>(p->d, out);
    return cudaGetLastError() == cudaSuccess ? QG_OK : QG_ERR_CUDA;
}
}  // namespace

extern "C" int qg_reparam_bc_vjp(qg_swm_plan* p, qg_plan* qp, float* y_bar, void* stream) {
    if (!p || !qp || !y_bar) return QG_ERR_NULL;
    if (p->desc.bc != QG_SWM_WALL) return QG_ERR_ARG;
    if (qg_plan_state_size(qp) != p->n / 3) return QG_ERR_SHAPE;
    cudaStream_t s = (cudaStream_t)stream;
    const int r = reparam_bc_project_vjp(p, qp, y_bar, p->stage, s);
    if (r != QG_OK) return r;
    return cudaMemcpyAsync(y_bar, p->stage, p->n * sizeof(float), cudaMemcpyDeviceToDevice, s) == cudaSuccess
               ? QG_OK
               : QG_ERR_CUDA;
}

extern "C" int64_t qg_reparam_step_vjp_workspace(const qg_swm_plan* p, int scheme) {
    const Tableau* tb = swm_scheme(scheme);
    if (!p || !tb) return -1;
    return (int64_t)(4 * tb->n) * p->n;
}

extern "C" int qg_reparam_step_vjp(qg_swm_plan* p, qg_plan* qp, const float* y0, const float* params, double dt,
                                   int scheme, float* y_bar, float* params_bar, float* work, void* stream) {
    if (!p || !qp || !y0 || !params || !y_bar || !params_bar || !work) return QG_ERR_NULL;
    const Tableau* tb = swm_scheme(scheme);
    if (!tb || !(dt == dt)) return QG_ERR_ARG;
    if (p->desc.bc != QG_SWM_WALL) return QG_ERR_ARG;
    if (qg_plan_state_size(qp) != p->n / 3) return QG_ERR_SHAPE;
    cudaStream_t s = (cudaStream_t)stream;
    const int ns = tb->n;
    const int64_t n = p->n;
    const int cgrid = (int)std::min<int64_t>(4096, (n + 255) / 256);
    // work: raw stage inputs Y_1 .. Y_{ns-1}, projected stage inputs Z_0 .. Z_{ns-1}, stage
    // derivatives K_0 .. K_{ns-2} (contiguous), their cotangents Kbar_0 .. Kbar_{ns-1}, and two
    // scratch states
    const float* Y[kMaxButcher];
    Y[0] = y0;
    for (int i = 1; i < ns; ++i) Y[i] = work + (int64_t)(i - 1) * n;
    float* Z = work + (int64_t)(ns - 1) * n;
    float* K = work + (int64_t)(2 * ns - 1) * n;
    float* Kb = work + (int64_t)(3 * ns - 2) * n;
    float* Zb = work + (int64_t)(4 * ns - 2) * n;
    float* T = work + (int64_t)(4 * ns - 1) * n;
    int r = QG_OK;
    cudaError_t e = cudaSuccess;
    for (int st = 0; st < ns && r == QG_OK; ++st) {
        r = reparam_bc_project(p, qp, Y[st], T, Z + st * n, s);
        if (r != QG_OK || st + 1 == ns) break;
        if (launch_stage(p, stage_args(p, Z + st * n, K + st * n, params, 0), s)) return QG_ERR_CUDA;
        Combine c{};
        for (int m = 0; m <= st; ++m) c.c[m] = (float)(dt * tb->a[st + 1][m]);
        k_swm_combine<<<cgrid, 256, 0, s>>>(const_cast<float*>(Y[st + 1]), y0, K, n, st + 1, c);
        if (cudaGetLastError() != cudaSuccess) return QG_ERR_CUDA;
    }
    if (r != QG_OK) return r;
    for (int st = 0; st < ns && !e; ++st) {
        k_swm_axpy<<<cgrid, 256, 0, s>>>(Kb + st * n, y_bar, (float)(dt * tb->b[st]), n, 1);
        e = cudaGetLastError();
    }
    if (!e) e = cudaMemsetAsync(p->pacc, 0, 4 * sizeof(double), s);
    for (int st = ns - 1; st >= 0 && !e; --st) {
        e = swm_vjp(p, Z + st * n, params, Kb + st * n, Zb, 0, s);
        if (e) break;
        r = reparam_bc_project_vjp(p, qp, Zb, T, s);
        if (r != QG_OK) return r;
        k_swm_axpy<<<cgrid, 256, 0, s>>>(y_bar, T, 1.f, n, 0);
        for (int m = 0; m < st; ++m)
            if (tb->a[st][m] != 0.0) k_swm_axpy<<<cgrid, 256, 0, s>>>(Kb + m * n, T, (float)(dt * tb->a[st][m]), n, 0);
        e = cudaGetLastError();
    }
    if (!e) {
        k_swm_pbar<<<1, 32, 0, s>>>(p->pacc, params_bar, 0);
        e = cudaGetLastError();
    }
    return e ? QG_ERR_CUDA : QG_OK;
}

extern "C" int qg_swm_status(qg_swm_plan* p, int* flags, void* stream) {
    if (!p) return QG_ERR_NULL;
    cudaStream_t s = (cudaStream_t)stream;
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, p->flags, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (!e) e = cudaMemsetAsync(p->flags, 0, sizeof(int), s);
    if (!e) e = cudaStreamSynchronize(s);
    if (e) return QG_ERR_CUDA;
    if (flags) *flags = h;
    return (h & 1) ? QG_ERR_NONFINITE : QG_OK;
}
