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

// Source of the stage-input value of field fld (0 = h, 1 = u, 2 = v) at (j, i) after the
// boundary rules (or as stored when !bc): its offset within the layer plane, or -1 where the
// wall rules set it to zero.
__device__ __forceinline__ int64_t src(const SwmDev& d, int fld, int j, int i, bool bc) {
    if (bc) {
        if (d.bc == QG_SWM_PERIODIC) {
            j = j == 0 ? d.Ny - 2 : (j == d.Ny - 1 ? 1 : j);
            i = i == 0 ? d.Nx - 2 : (i == d.Nx - 1 ? 1 : i);
        } else {
            if (fld == 1 && (i == 0 || i >= d.Nx - 2)) return -1;
            if (fld == 2 && (j == 0 || j >= d.Ny - 2)) return -1;
            if (fld != 2) j = min(max(j, 1), d.Ny - 2);
            if (fld != 1) i = min(max(i, 1), d.Nx - 2);
        }
    }
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

// PV, face mass fluxes, kinetic energy and the pressure sum of one point of the haloed tile
// (row r, column c; T-cell (jj, ii)).  Each is formed where some own cell of the tile reads it.
template <bool INT>
__device__ __forceinline__ void derive_point(StageTables& t, const SwmDev& d, float g, int r, int c, int jj, int ii,
                                             float& q, float& uh, float& vh, float& ke, float& p) {
    const int e = r * kStX + c;
    q = 0.f, uh = 0.f, vh = 0.f, ke = 0.f;
    if (INT || (jj >= 1 && jj <= d.Ny - 2 && ii >= 1 && ii <= d.Nx - 2)) {
        if (r < kStY - 1 && c < kStX - 1) {
            const float zeta = (t.v[e + 1] - t.v[e]) * d.idx - (t.u[e + kStX] - t.u[e]) * d.idy;
            const float hX = 0.25f * (t.h[e] + t.h[e + 1] + t.h[e + kStX] + t.h[e + kStX + 1]);
            q = (zeta + __ldg(d.fx + jj)) / hX;
        }
        if (c < kStX - 1) uh = 0.5f * (t.h[e] + t.h[e + 1]) * t.u[e];
        if (r < kStY - 1) vh = 0.5f * (t.h[e] + t.h[e + kStX]) * t.v[e];
        if (r > 0 && c > 0) {
            const float ua = t.u[e], ub = t.u[e - 1], va = t.v[e], vb = t.v[e - kStX];
            ke = 0.25f * (ua * ua + ub * ub + va * va + vb * vb);
        }
    }
    p = fmaf(g, t.h[e], p);
    t.q[e] = q;
    t.uh[e] = uh;
    t.vh[e] = vh;
    t.ke[e] = ke;
    t.p[e] = p;
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
    bool bad = false;
    float po = 0.f, ph = 0.f;  // cumulative pressure at the own and the halo cell
    for (int k = 0; k < d.nl; ++k) {
        const int64_t lo = k * plane;
        float vo[3][NS + 1], vh[3][NS + 1], yo3[3], yh3[3];
        if (mine) load_point<NS, INT>(d, a, field, lo, j, i, vo);
        if (halo) load_point<NS, INT>(d, a, field, lo, j0 + hr, i0 + hc, vh);
        if (mine) store_input<NS>(t, a, eo, vo, yo3);
        if (halo) store_input<NS>(t, a, he, vh, yh3);
        __syncthreads();
        const float g = __ldg(d.gp + k);
        float qo = 0.f, uho = 0.f, vho = 0.f, keo = 0.f, x0, x1, x2, x3;
        if (mine) derive_point<INT>(t, d, g, threadIdx.y + 1, threadIdx.x + 1, j, i, qo, uho, vho, keo, po);
        if (halo) derive_point<INT>(t, d, g, hr, hc, j0 + hr, i0 + hc, x0, x1, x2, x3, ph);
        __syncthreads();
        if (mine) {
            const bool top = k == 0, bottom = k == d.nl - 1;
            const int e = eo;
            const float uc = yo3[1], vc = yo3[2];
            float dh = 0.f;
            float du = (top ? tau0 * __ldg(d.wx + j) * d.invH0 : 0.f) - (bottom ? kappa * uc : 0.f);
            float dv = bottom ? -kappa * vc : 0.f;
            if (in) {
                const float hc0 = yo3[0], uw = t.u[e - 1], vs = t.v[e - kStX];
                const float fe = uc * (uc > 0.f ? hc0 : t.h[e + 1]);
                const float fw = uw * (uw > 0.f ? t.h[e - 1] : hc0);
                const float gn = vc * (vc > 0.f ? hc0 : t.h[e + kStX]);
                const float gs = vs * (vs > 0.f ? t.h[e - kStX] : hc0);
                dh = -((fe - fw) * d.idx + (gn - gs) * d.idy);
                const float qU = 0.5f * (qo + t.q[e - kStX]);
                const float qV = 0.5f * (qo + t.q[e - 1]);
                const float vhU = 0.25f * (vho + t.vh[e + 1] + t.vh[e - kStX] + t.vh[e - kStX + 1]);
                const float uhV = 0.25f * (uho + t.uh[e - 1] + t.uh[e + kStX] + t.uh[e + kStX - 1]);
                const float Pc = keo + po, Pe = t.ke[e + 1] + t.p[e + 1];
                const float Pn = t.ke[e + kStX] + t.p[e + kStX];
                const float lu =
                    (t.u[e + 1] - 2.f * uc + uw) * d.idx2 + (t.u[e + kStX] - 2.f * uc + t.u[e - kStX]) * d.idy2;
                const float lv =
                    (t.v[e + 1] - 2.f * vc + t.v[e - 1]) * d.idx2 + (t.v[e + kStX] - 2.f * vc + vs) * d.idy2;
                du += qU * vhU - (Pe - Pc) * d.idx + nu * lu;
                dv += -qV * uhV - (Pn - Pc) * d.idy + nu * lv;
            }
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
    int* flags = nullptr;
    int64_t n = 0;            // floats of one state
    int device = 0;
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
    if (!e) e = cudaMalloc(&p->proj, p->n * sizeof(float));
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
    for (cudaGraphExec_t x : {p->g8, p->g1})
        if (x) cudaGraphExecDestroy(x);
    for (auto& v : p->ev)
        for (auto& pr : v) {
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
    if (p->cap) cudaStreamDestroy(p->cap);
    for (void* a : {(void*)p->consts, (void*)p->stage, (void*)p->K, (void*)p->params, (void*)p->proj,
                    (void*)p->flags})
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

extern "C" int qg_swm_step(qg_swm_plan* p, float* state, const float* params, double dt, int n_steps, int scheme,
                           int flags, void* stream) {
    if (!p || !state || !params) return QG_ERR_NULL;
    if (n_steps < 0 || (flags & ~QG_STEP_APPLY_BC) || !(dt == dt)) return QG_ERR_ARG;
    const Tableau* tb = swm_tableau(scheme);
    if (!tb) return QG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = cudaMemcpyAsync(p->params, params, 3 * sizeof(float), cudaMemcpyDeviceToDevice, s);
    if (!e && (flags & QG_STEP_APPLY_BC)) {
        k_swm_bc<<<swm_grid(p->d), dim3(kSwTX, kSwTY), 0, s>>>(p->d, state);
        e = cudaGetLastError();
    }
    if (e || n_steps == 0) return e ? QG_ERR_CUDA : QG_OK;
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
