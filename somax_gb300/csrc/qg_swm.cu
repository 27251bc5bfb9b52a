// Multilayer shallow-water right-hand side (MultilayerShallowWater2D.vector_field,
// somax/_src/models/swm/multilayer.py:150-200) and its constant-step integration.
//
// State layout: one packed float32 array (3, nl, Ny, Nx) = h, u, v per layer, row-major, one
// ghost ring; h at T points (cell centres), u at U points (east faces), v at V points (north
// faces).  The C-grid operators are finitevolx's, restated: each writes the interior and leaves
// the ring zero, the mass flux is first-order upwind on every face an interior cell needs.
//
// k_swm_rhs: one thread per (j, i) column computes dh, du, dv of every layer in one pass, with
// the boundary rules applied on read when asked (periodic wrap, or the wall rules: u = 0 on the
// west ring, the east wall face and the east ring; v = 0 on the south ring, the north wall face
// and the north ring; free slip and zero gradient elsewhere on the ring).  Per layer k:
//   dh = -div(h u) (upwind h on the faces)
//   q  = (zeta + f) / h at X points (interior), f and h interpolated from T points
//   du = X_to_U(q) V_to_U(h_V v) - d_x P + [k = 0] tau0 wind_x / H0 + nu lap u - [bottom] kappa u
//   dv = -X_to_V(q) U_to_V(h_U u) - d_y P + nu lap v - [bottom] kappa v
//   P  = KE + sum_{l <= k} g'_l h_l, KE = (U_to_T(u^2) + V_to_T(v^2)) / 2 (interior)
// The thread walks the layers once, carrying the cumulative pressure at its T point and at the
// east and north neighbours.  The fields stay in L1 / L2 between the neighbouring threads' reads,
// so HBM sees each input once and each output once: 24 B per cell and layer.
//
// k_swm_combine: y = y0 + sum_s c_s k_s over the packed state (Butcher-form stage inputs and
// the step update).
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
    float gp[QG_MAX_LAYERS];
    float invH0;
    int bc;           // QG_SWM_PERIODIC / QG_SWM_WALL
    const float* fx;  // f interpolated to the X rows: (f[j] + f[j + 1]) / 2
    const float* wx;  // wind pattern at the T rows
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

__global__ void __launch_bounds__(kSwTX * kSwTY) k_swm_rhs(SwmDev d, const float* __restrict__ y,
                                                            float* __restrict__ dy, const float* __restrict__ params,
                                                            int bc, int* flags) {
    const int i = blockIdx.x * kSwTX + threadIdx.x;
    const int j = blockIdx.y * kSwTY + threadIdx.y;
    if (i >= d.Nx || j >= d.Ny) return;
    const float nu = params[0], kappa = params[1], tau0 = params[2];
    const int64_t plane = (int64_t)d.Ny * d.Nx, field = plane * d.nl;
    const int64_t o = (int64_t)j * d.Nx + i;
    const bool in = j >= 1 && j <= d.Ny - 2 && i >= 1 && i <= d.Nx - 2;
    const bool use_bc = bc != 0;
    float pc = 0.f, pe = 0.f, pn = 0.f;  // cumulative pressure at (j, i), (j, i + 1), (j + 1, i)
    bool bad = false;
    for (int k = 0; k < d.nl; ++k) {
        const float* h = y + k * plane;
        const float* u = y + field + k * plane;
        const float* v = y + 2 * field + k * plane;
        auto H = [&](int a, int b) { return ld(h, d, 0, a, b, use_bc); };
        auto U = [&](int a, int b) { return ld(u, d, 1, a, b, use_bc); };
        auto V = [&](int a, int b) { return ld(v, d, 2, a, b, use_bc); };
        auto inside = [&](int a, int b) { return a >= 1 && a <= d.Ny - 2 && b >= 1 && b <= d.Nx - 2; };
        const float g = d.gp[k];
        pc = fmaf(g, H(j, i), pc);
        if (i + 1 < d.Nx) pe = fmaf(g, H(j, i + 1), pe);
        if (j + 1 < d.Ny) pn = fmaf(g, H(j + 1, i), pn);
        const bool top = k == 0, bottom = k == d.nl - 1;
        const float uc = U(j, i), vc = V(j, i);
        float dh = 0.f;
        float du = (top ? tau0 * d.wx[j] * d.invH0 : 0.f) - (bottom ? kappa * uc : 0.f);
        float dv = bottom ? -kappa * vc : 0.f;
        if (in) {
            // mass: upwind fluxes on the four faces of the cell
            const float hc = H(j, i);
            const float uw = U(j, i - 1), vs = V(j - 1, i);
            const float fe = uc * (uc > 0.f ? hc : H(j, i + 1));
            const float fw = uw * (uw > 0.f ? H(j, i - 1) : hc);
            const float gn = vc * (vc > 0.f ? hc : H(j + 1, i));
            const float gs = vs * (vs > 0.f ? H(j - 1, i) : hc);
            dh = -((fe - fw) * d.idx + (gn - gs) * d.idy);
            // PV at the X points around the cell (interior write: zero on the ring)
            auto qX = [&](int a, int b) {
                if (!inside(a, b)) return 0.f;
                const float zeta = (V(a, b + 1) - V(a, b)) * d.idx - (U(a + 1, b) - U(a, b)) * d.idy;
                const float hX = 0.25f * (H(a, b) + H(a, b + 1) + H(a + 1, b) + H(a + 1, b + 1));
                return (zeta + d.fx[a]) / hX;
            };
            auto uh = [&](int a, int b) { return inside(a, b) ? 0.5f * (H(a, b) + H(a, b + 1)) * U(a, b) : 0.f; };
            auto vh = [&](int a, int b) { return inside(a, b) ? 0.5f * (H(a, b) + H(a + 1, b)) * V(a, b) : 0.f; };
            auto ke = [&](int a, int b) {
                if (!inside(a, b)) return 0.f;
                const float ua = U(a, b), ub = U(a, b - 1), va = V(a, b), vb = V(a - 1, b);
                return 0.25f * (ua * ua + ub * ub + va * va + vb * vb);
            };
            const float q0 = qX(j, i);
            const float qU = 0.5f * (q0 + qX(j - 1, i));
            const float qV = 0.5f * (q0 + qX(j, i - 1));
            const float vhU = 0.25f * (vh(j, i) + vh(j, i + 1) + vh(j - 1, i) + vh(j - 1, i + 1));
            const float uhV = 0.25f * (uh(j, i) + uh(j, i - 1) + uh(j + 1, i) + uh(j + 1, i - 1));
            const float Pc = ke(j, i) + pc, Pe = ke(j, i + 1) + pe, Pn = ke(j + 1, i) + pn;
            const float lu = (U(j, i + 1) - 2.f * uc + uw) * d.idx2 + (U(j + 1, i) - 2.f * uc + U(j - 1, i)) * d.idy2;
            const float lv = (V(j, i + 1) - 2.f * vc + V(j, i - 1)) * d.idx2 + (V(j + 1, i) - 2.f * vc + vs) * d.idy2;
            du += qU * vhU - (Pe - Pc) * d.idx + nu * lu;
            dv += -qV * uhV - (Pn - Pc) * d.idy + nu * lv;
        }
        bad |= !isfinite(dh) || !isfinite(du) || !isfinite(dv);
        dy[k * plane + o] = dh;
        dy[field + k * plane + o] = du;
        dy[2 * field + k * plane + o] = dv;
    }
    if (bad && flags) atomicOr(flags, 1);
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
    int* flags = nullptr;
    int64_t n = 0;            // floats of one state
    int device = 0;
};

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
    for (int k = 0; k < s.n_layers; ++k) d.gp[k] = (float)s.g_prime[k];
    d.invH0 = (float)(1.0 / s.H[0]);
    d.bc = s.bc;
    p->n = (int64_t)3 * d.nl * d.Ny * d.Nx;
    // f at the X rows and the wind pattern at the T rows (f(y) = f0 + beta (y - Ly / 2),
    // y_j = j dy; tau_x = -cos(2 pi y / Ly) or -cos(pi y / Ly)), rounded once from float64
    std::vector<float> c(2 * (size_t)d.Ny);
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
    if (!e) e = cudaMalloc(&p->flags, 16);
    if (!e) e = cudaMemset(p->flags, 0, 16);
    if (e) {
        qg_swm_destroy(p);
        return QG_ERR_CUDA;
    }
    d.fx = p->consts;
    d.wx = p->consts + d.Ny;
    *out = p;
    return QG_OK;
}

extern "C" void qg_swm_destroy(qg_swm_plan* p) {
    if (!p) return;
    cudaDeviceSynchronize();
    for (void* a : {(void*)p->consts, (void*)p->stage, (void*)p->K, (void*)p->flags})
        if (a) cudaFree(a);
    delete p;
}

extern "C" int64_t qg_swm_state_size(const qg_swm_plan* p) { return p ? p->n : -1; }

extern "C" int qg_swm_rhs(qg_swm_plan* p, const float* state, float* tend, const float* params, int flags,
                          void* stream) {
    if (!p || !state || !tend || !params) return QG_ERR_NULL;
    if (flags & ~QG_RHS_APPLY_BC) return QG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    k_swm_rhs<<<swm_grid(p->d), dim3(kSwTX, kSwTY), 0, s>>>(p->d, state, tend, params, flags & QG_RHS_APPLY_BC,
                                                             p->flags);
    return cudaGetLastError() == cudaSuccess ? QG_OK : QG_ERR_CUDA;
}

extern "C" int qg_swm_apply_bc(qg_swm_plan* p, float* state, void* stream) {
    if (!p || !state) return QG_ERR_NULL;
    k_swm_bc<<<swm_grid(p->d), dim3(kSwTX, kSwTY), 0, (cudaStream_t)stream>>>(p->d, state);
    return cudaGetLastError() == cudaSuccess ? QG_OK : QG_ERR_CUDA;
}

extern "C" int qg_swm_step(qg_swm_plan* p, float* state, const float* params, double dt, int n_steps, int scheme,
                           int flags, void* stream) {
    if (!p || !state || !params) return QG_ERR_NULL;
    if (n_steps < 0 || (flags & ~QG_STEP_APPLY_BC) || !(dt == dt)) return QG_ERR_ARG;
    const Tableau* tb = swm_tableau(scheme);
    if (!tb) return QG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const dim3 g = swm_grid(p->d), b(kSwTX, kSwTY);
    const int cgrid = (int)std::min<int64_t>(4096, (p->n + 255) / 256);
    if (flags & QG_STEP_APPLY_BC) k_swm_bc<<<g, b, 0, s>>>(p->d, state);
    for (int step = 0; step < n_steps; ++step) {
        for (int st = 0; st < tb->n; ++st) {
            const float* yin = state;
            if (st > 0) {
                Combine c{};
                for (int j = 0; j < st; ++j) c.c[j] = (float)(dt * tb->a[st][j]);
                k_swm_combine<<<cgrid, 256, 0, s>>>(p->stage, state, p->K, p->n, st, c);
                yin = p->stage;
            }
            k_swm_rhs<<<g, b, 0, s>>>(p->d, yin, p->K + st * p->n, params, 1, p->flags);
        }
        Combine c{};
        for (int j = 0; j < tb->n; ++j) c.c[j] = (float)(dt * tb->b[j]);
        k_swm_combine<<<cgrid, 256, 0, s>>>(state, state, p->K, p->n, tb->n, c);
    }
    return cudaGetLastError() == cudaSuccess ? QG_OK : QG_ERR_CUDA;
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
