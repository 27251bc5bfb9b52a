// Host side of libqgcore: plan construction (FP64 modal matrices, DST-I matrices and
// eigenvalues, grids of tiles), the C-ABI entry points and their launch sequences, CUDA
// graph capture of a whole time step, and per-kernel event timing.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <new>
#include <vector>

#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {
cudaError_t gemm_tc_init();
int gemm_tc_tile_n(int precision);
}  // namespace qg

using namespace qg;

namespace {

// sweep item lists: strip heights 16, 32, 64 of the one-layer-per-lane sweep, then of the
// layer-per-warp sweep
constexpr int kSweepLists = 6;
constexpr int kSweepGroups = kMaxLayers * kLSweepClasses;

// ---------------------------------------------------------------------------------------
// Small dense linear algebra in double (nl <= 8)
// ---------------------------------------------------------------------------------------

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (row-major).  On return
// w holds the eigenvalues (ascending) and V's columns the orthonormal eigenvectors.
void jacobi_eigh(int n, const double* Ain, double* w, double* V) {
    double A[kMaxLayers * kMaxLayers];
    std::memcpy(A, Ain, sizeof(double) * n * n);
    for (int i = 0; i < n * n; ++i) V[i] = 0.0;
    for (int i = 0; i < n; ++i) V[i * n + i] = 1.0;
    for (int sweep = 0; sweep < 100; ++sweep) {
        double off = 0.0, tot = 0.0;
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j) {
                tot += A[i * n + j] * A[i * n + j];
                if (i != j) off += A[i * n + j] * A[i * n + j];
            }
        if (off <= 1e-30 * tot || off == 0.0) break;
        for (int p = 0; p < n - 1; ++p)
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[p * n + q];
                if (apq == 0.0) continue;
                const double theta = (A[q * n + q] - A[p * n + p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {  // A <- A J
                    const double akp = A[k * n + p], akq = A[k * n + q];
                    A[k * n + p] = c * akp - s * akq;
                    A[k * n + q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {  // A <- J^T A
                    const double apk = A[p * n + k], aqk = A[q * n + k];
                    A[p * n + k] = c * apk - s * aqk;
                    A[q * n + k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {  // V <- V J
                    const double vkp = V[k * n + p], vkq = V[k * n + q];
                    V[k * n + p] = c * vkp - s * vkq;
                    V[k * n + q] = s * vkp + c * vkq;
                }
            }
    }
    // sort ascending
    int idx[kMaxLayers];
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::sort(idx, idx + n, [&](int a, int b) { return A[a * n + a] < A[b * n + b]; });
    double Vs[kMaxLayers * kMaxLayers];
    for (int c = 0; c < n; ++c) {
        w[c] = A[idx[c] * n + idx[c]];
        for (int r = 0; r < n; ++r) Vs[r * n + c] = V[r * n + idx[c]];
    }
    std::memcpy(V, Vs, sizeof(double) * n * n);
}

}  // namespace

namespace qg {

// Layered QG coupling A = diag(1/H) M with M symmetric tridiagonal (the stretching
// operator of finitevolx build_coupling_matrix, transforms.py:192).  Its right
// eigenvectors are R = diag(H^-1/2) V with V the eigenvectors of the symmetric
// diag(H^-1/2) M diag(H^-1/2); Cl2m = R^-1 = V^T diag(H^1/2).
void vertical_modes(const qg_member_desc& d, double* Cl2m, double* Cm2l, double* lam) {
    const int n = d.n_layers;
    double Msym[kMaxLayers * kMaxLayers] = {0};
    if (n == 1) {
        Msym[0] = 1.0 / d.g_prime[0];
    } else {
        for (int k = 0; k < n; ++k) {
            double dk = (k < n - 1) ? 1.0 / d.g_prime[k + 1] : 0.0;
            dk += (k == 0) ? 1.0 / d.g_prime[0] : 0.0;
            if (k > 0) dk += 1.0 / d.g_prime[k];
            Msym[k * n + k] = dk;
            if (k < n - 1) Msym[k * n + k + 1] = Msym[(k + 1) * n + k] = -1.0 / d.g_prime[k + 1];
        }
    }
    double S[kMaxLayers * kMaxLayers], w[kMaxLayers], V[kMaxLayers * kMaxLayers];
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) S[i * n + j] = Msym[i * n + j] / std::sqrt(d.H[i] * d.H[j]);
    jacobi_eigh(n, S, w, V);
    for (int i = 0; i < n; ++i)
        for (int m = 0; m < n; ++m) {
            Cm2l[i * n + m] = V[i * n + m] / std::sqrt(d.H[i]);
            Cl2m[m * n + i] = V[i * n + m] * std::sqrt(d.H[i]);
        }
    if (d.eigs_mode == QG_EIGS_REFERENCE) {
        // jnp.linalg.eigh symmetrises its input: eigenvalues of (A + A^T)/2
        double As[kMaxLayers * kMaxLayers], Vr[kMaxLayers * kMaxLayers];
        for (int i = 0; i < n; ++i)
            for (int j = 0; j < n; ++j)
                As[i * n + j] = 0.5 * (Msym[i * n + j] / d.H[i] + Msym[j * n + i] / d.H[j]);
        jacobi_eigh(n, As, w, Vr);
    }
    for (int m = 0; m < n; ++m) lam[m] = d.f0 * d.f0 * w[m];
}

int round_up(int v, int m) { return (v + m - 1) / m * m; }

int validate_member(const qg_member_desc& d) {
    if (d.nx < 1 || d.ny < 1 || d.n_layers < 1 || d.n_layers > QG_MAX_LAYERS) return QG_ERR_SHAPE;
    if ((int64_t)(d.nx + 2) * (d.ny + 2) > (1LL << 28)) return QG_ERR_SHAPE;
    if (d.barotropic && d.n_layers != 1) return QG_ERR_SHAPE;
    if (!(d.Lx > 0) || !(d.Ly > 0)) return QG_ERR_ARG;
    if (d.wind_profile != QG_WIND_DOUBLEGYRE && d.wind_profile != QG_WIND_SINGLE) return QG_ERR_ARG;
    if (d.eigs_mode != QG_EIGS_CONSISTENT && d.eigs_mode != QG_EIGS_REFERENCE) return QG_ERR_ARG;
    if (!d.has_modes && !d.barotropic)
        for (int l = 0; l < d.n_layers; ++l)
            if (!(d.H[l] > 0) || !(d.g_prime[l] > 0)) return QG_ERR_ARG;
    return QG_OK;
}

// Geometry, finite-difference constants and modal matrices of one member (the device
// pointers and offsets are left zero for the caller to fill).
void member_constants(const qg_member_desc& d, MemberDev& M, double* Cl2m, double* Cm2l, double* lam) {
    std::memset(&M, 0, sizeof(M));
    M.nl = d.n_layers;
    M.Ny = d.ny + 2;
    M.Nx = d.nx + 2;
    M.Px = round_up(M.Nx, 32);
    M.Py = round_up(M.Ny, 32);
    M.barotropic = d.barotropic;
    const double dx = d.Lx / d.nx, dy = d.Ly / d.ny;
    M.dx = (float)dx;
    M.dy = (float)dy;
    M.inv_dx2 = (float)(1.0 / (dx * dx));
    M.inv_dy2 = (float)(1.0 / (dy * dy));
    M.inv_12dxdy = (float)(1.0 / (12.0 * dx * dy));
    M.beta_12dx = (float)(d.beta / (12.0 * dx));
    M.invH0 = d.barotropic ? 1.f : (float)(1.0 / d.H[0]);
    M.f0 = (float)d.f0;
    for (int l = 0; l < d.n_layers && !d.barotropic; ++l) M.H[l] = (float)d.H[l];
    const int n = d.n_layers;
    if (d.barotropic) {
        Cl2m[0] = Cm2l[0] = 1.0;
        lam[0] = 0.0;
    } else if (d.has_modes) {
        for (int k = 0; k < n * n; ++k) {
            Cl2m[k] = d.Cl2m[k];
            Cm2l[k] = d.Cm2l[k];
        }
        for (int k = 0; k < n; ++k) lam[k] = d.lambdas[k];
    } else {
        vertical_modes(d, Cl2m, Cm2l, lam);
    }
    for (int r = 0; r < n; ++r) {
        for (int c = 0; c < n; ++c) {
            M.Cl2m[r * kMaxLayers + c] = (float)Cl2m[r * n + c];
            M.Cm2l[r * kMaxLayers + c] = (float)Cm2l[r * n + c];
        }
        M.lam[r] = (float)lam[r];
    }
}

}  // namespace qg

namespace {

// Orthonormal DST-I matrix (n x n, pitch ld): sqrt(2/(n+1)) sin(pi (i+1)(j+1)/(n+1)),
// the argument reduced modulo 2(n+1) for accuracy.
void dst_matrix(int n, int ld, std::vector<float>& out) {
    out.assign((size_t)n * ld, 0.f);
    const double s = std::sqrt(2.0 / (n + 1));
    const long long per = 2LL * (n + 1);
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) {
            const long long k = ((long long)(i + 1) * (j + 1)) % per;
            out[(size_t)i * ld + j] = (float)(s * std::sin(M_PI * (double)k / (n + 1)));
        }
}

// Eigenvalues of the 3-point second difference with Dirichlet zeros at -1 and n:
// (2 cos(pi k/(n+1)) - 2)/d^2 = -4 sin^2(pi k / (2(n+1))) / d^2.
void dst_eigs(int n, double d, std::vector<float>& out) {
    out.resize(n);
    for (int k = 1; k <= n; ++k) {
        const double sn = std::sin(M_PI * k / (2.0 * (n + 1)));
        out[k - 1] = (float)(-4.0 * sn * sn / (d * d));
    }
}

const char* kErrStr[] = {"ok", "null pointer", "bad shape", "CUDA error", "non-finite value",
                         "device wait timed out", "bad argument", "unsupported",
                         "member exceeds a size limit (static scratch, or land boundary points)"};

}  // namespace

// Captured steps of qg_step: one step, and kGraphSteps steps in one graph, so that the
// kernels of consecutive steps chain with programmatic dependent launch instead of draining
// the GPU at every graph boundary.
constexpr int kGraphSteps = 8;
struct StepGraph {
    cudaGraphExec_t exec = nullptr;    // one step
    cudaGraphExec_t exec_k = nullptr;  // kGraphSteps steps
    double dt = 0.0;
    int scheme = -1;
};

// The captured launch sequence of one qg_step_vjp call and the arguments it was captured with
// (replayed while they repeat).
struct VjpGraph {
    cudaGraphExec_t exec = nullptr;
    const void* ptr[5] = {};  // y0, params, y_bar, params_bar, work
    double dt = 0.0;
    int scheme = -1;
};

struct qg_plan {
    int n_members = 0;
    qg_options opts{};
    std::vector<qg_member_desc> desc;
    std::vector<MemberDev> mh;  // host copy of member constants (device pointers filled)
    MemberDev* md = nullptr;    // device
    int max_nl = 1;
    int64_t state_size = 0, xplane = 0, yplane = 0, total_layers = 0;
    std::vector<int64_t> member_off;
    // tiles
    StencilTile* st_tiles = nullptr;
    int n_st = 0;
    GemmTile* gx_tiles = nullptr;  // passes with A in x-row planes (G1, G4)
    GemmTile* gy_tiles = nullptr;  // passes with A in y-row planes (G2, G3)
    int n_gx = 0, n_gy = 0;
    // tensor-core tile lists for each candidate output tile width (kGemmBN); the autotuner
    // keeps the fastest (wide tiles for large members, narrow ones spread small members)
    GemmTile* gx_v[5] = {};
    GemmTile* gy_v[5] = {};
    int n_gx_v[5] = {}, n_gy_v[5] = {};
    int n_bn = 1, bn_sel = 0;
    float tune_gemm_ms[5] = {-1.f, -1.f, -1.f, -1.f, -1.f};
    // cluster-resident stepping (qg_cluster.cu): CTAs per member's cluster (0: not possible),
    // its dynamic shared memory, the members' layer count, whether qg_step uses it, and the
    // autotuner's times of four SSP-RK3 steps (multi-launch, cluster)
    int cl_C = 0;
    size_t cl_smem = 0;
    int cl_nl = 0;
    bool cl_use = false;
    float tune_engine_ms[2] = {-1.f, -1.f};
    // device memory: x-row planes XA (modal operand), XB (U, the divided spectrum), XC
    // (psi_hat), XQ (FP32 modal rhs for refinement), S0 (state), S1/S2 (stage inputs); y-row
    // planes YA (T1) and YB (V), the outputs of the x-contracting passes
    std::vector<void*> allocs;
    float *XA = nullptr, *XB = nullptr, *XC = nullptr, *XQ = nullptr, *YA = nullptr, *YB = nullptr;
    float *S0 = nullptr, *S1 = nullptr, *S2 = nullptr;
    float* K = nullptr;  // Butcher-form stage derivatives (kMaxStages caller-packed fields)
    float* params = nullptr;  // plan-owned copy of the params (graph-stable)
    // masked members: capacitance work items (one per mode and block of rows of C^-1)
    CapItem* cap_items = nullptr;
    int n_cap = 0;
    size_t cap_smem = 0;
    int* flags = nullptr;
    double* diag_acc = nullptr;
    void* stats_acc = nullptr;  // qg_state_stats accumulators (32 bytes)
    double* vjp_acc = nullptr;  // parameter cotangents of qg_rhs_vjp (QG_NPARAMS per member)
    int op_fmt = FMT_F32;
    void* tc_maps = nullptr;  // TMA descriptors of the tensor-core GEMMs
    void* st_maps = nullptr;  // TMA descriptors of the stencil halo boxes
    unsigned* bar = nullptr;  // grid barrier words of the persistent kernel (count, generation)
    int n_sm = 0;
    int st_large = 0;         // stencil tile shape in use: 0 = 32 x 8, 1 = 64 x 16
    int st_grid = 1;          // CTAs of a stencil launch (tiles round-robin over them)
    // both stencil tile shapes are prepared; the autotuner (or a size rule) picks one
    StencilTile* st_tiles_v[2] = {nullptr, nullptr};
    int n_st_v[2] = {0, 0};
    void* st_maps_v[2] = {nullptr, nullptr};
    float tune_ms[QG_STENCIL_VARIANTS] = {-1.f, -1.f, -1.f, -1.f, -1.f, -1.f, -1.f, -1.f};
    // column-sweep stencils: item lists of the one-layer-per-lane sweep (v = 0, 1, 2) and the
    // layer-per-warp sweep (v = 3, 4, 5) for 16-, 32- and 64-row strips; sw_sel = the one the
    // multi-launch path runs (-1: the tile stencil)
    SweepItem* sw_items_v[kSweepLists] = {};
    int n_sw_v[kSweepLists] = {};
    // items of each list grouped by layer count and strip class: group k * kLSweepClasses + c
    // (k + 1 layers, class c; always class 0 for the one-layer-per-lane sweep) at offset sw_off
    int sw_off[kSweepLists][kSweepGroups] = {};
    int sw_cnt[kSweepLists][kSweepGroups] = {};
    int sw_sel = -1;
    int sw_grid[kSweepGroups] = {};
    PersistArgs pa{};         // constant part of the tensor-core launches' arguments
    // graphs
    cudaStream_t cap = nullptr;
    // the layer-per-warp sweep's (layer count, strip class) launches are independent: they run
    // as parallel branches on these streams (forked from and joined into the stage's stream)
    static constexpr int kSide = 4;
    cudaStream_t side[kSide] = {};
    cudaEvent_t fork_ev = nullptr;
    cudaEvent_t join_ev[kSweepGroups] = {};
    bool fork_on = true;  // qg_plan_set_parallel_sweep: 0 launches the groups one after another
    StepGraph graph;
    VjpGraph vjp_graph;
    // profiling
    bool profiling = false;
    std::vector<std::pair<cudaEvent_t, cudaEvent_t>> ev[QG_K_COUNT];
    size_t ev_used[QG_K_COUNT] = {0, 0, 0, 0, 0};
    int device = 0;
};

namespace {

PFN_cuTensorMapEncodeTiled_v12000 g_encode = nullptr;

cudaError_t tmap_init() {
    if (g_encode) return cudaSuccess;
    void* fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    cudaError_t e = cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q);
    if (e || q != cudaDriverEntryPointSuccess || !fn) return cudaErrorNotSupported;
    g_encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
    return cudaSuccess;
}

template <typename T>
cudaError_t dalloc(qg_plan* p, T** ptr, size_t bytes) {
    void* v = nullptr;
    cudaError_t e = cudaMalloc(&v, std::max<size_t>(bytes, 16));
    if (e != cudaSuccess) return e;
    cudaMemsetAsync(v, 0, std::max<size_t>(bytes, 16));
    p->allocs.push_back(v);
    *ptr = static_cast<T*>(v);
    return cudaSuccess;
}

template <typename T>
cudaError_t upload(qg_plan* p, T** dst, const std::vector<T>& src) {
    cudaError_t e = dalloc(p, dst, src.size() * sizeof(T));
    if (e != cudaSuccess) return e;
    return cudaMemcpy(*dst, src.data(), src.size() * sizeof(T), cudaMemcpyHostToDevice);
}

// Run `launch` bracketed by profiling events of class k when profiling is on.
template <typename F>
cudaError_t timed(qg_plan* p, int k, cudaStream_t s, F&& launch) {
    if (!p->profiling) return launch();
    auto& v = p->ev[k];
    if (p->ev_used[k] == v.size()) {
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        v.emplace_back(a, b);
    }
    auto& pr = v[p->ev_used[k]++];
    cudaEventRecord(pr.first, s);
    cudaError_t e = launch();
    cudaEventRecord(pr.second, s);
    return e;
}

// Kernels may overlap their prologue with the predecessor (programmatic dependent launch)
// except while profiling, where events separate every launch.
bool use_pdl(const qg_plan* p) { return !p->profiling; }

GemmArgs gemm_args(qg_plan* p, int pass, const void* A, void* C, int a_fmt, int c_fmt, int acc) {
    GemmArgs g{};
    g.members = p->md;
    g.xplane = p->xplane;
    g.yplane = p->yplane;
    g.tiles = pass_xin(pass) ? p->gx_tiles : p->gy_tiles;
    g.pass = pass;
    g.A = A;
    g.C = C;
    g.a_fmt = a_fmt;
    g.c_fmt = c_fmt;
    g.accumulate = acc;
    g.tc_maps = p->tc_maps;
    g.flags = p->flags;
    return g;
}

// Schedule of a tensor-core GEMM pass's tiles over its G = SM-count CTAs (CTA b takes tiles
// b, b + G, b + 2G, ... of the list, one after another).  The output tiles of one M-tile (a
// member's N-tiles: 258-wide members need two 144-wide ones) read the same A rows, so they stay
// together on one CTA, in sequence, while the A rows it just streamed are still in L2.  The
// M-tiles go to CTAs longest first, each to the CTA with the least work so far (cost of a
// tile: its k-blocks plus a fixed epilogue share), which evens out the CTAs' totals (the
// pass lasts as long as its busiest CTA); CTAs with fewer tiles get padding entries
// (member -1) that every role of the kernel skips.  Lists shorter than two tiles per CTA keep
// their order.  Only the order changes: every tile is computed once.
std::vector<GemmTile> schedule_tiles(const std::vector<GemmTile>& in, int G, const std::vector<int>& kdim) {
    if (G < 1 || (int64_t)in.size() < 2 * (int64_t)G) return in;
    std::vector<std::vector<GemmTile>> rows;  // tiles of one (member, mt), nt ascending
    for (const GemmTile& t : in) {
        if (!rows.empty() && rows.back()[0].member == t.member && rows.back()[0].mt == t.mt)
            rows.back().push_back(t);
        else
            rows.push_back({t});
    }
    std::vector<double> cost(rows.size());
    for (size_t r = 0; r < rows.size(); ++r)
        cost[r] = rows[r].size() * ((kdim[rows[r][0].member] + 63) / 64 + 1.5);
    std::vector<size_t> order(rows.size());
    for (size_t r = 0; r < order.size(); ++r) order[r] = r;
    std::stable_sort(order.begin(), order.end(), [&](size_t a, size_t b) { return cost[a] > cost[b]; });
    std::vector<double> load(G, 0.0);
    std::vector<std::vector<GemmTile>> seq(G);
    for (size_t r : order) {
        const int b = (int)(std::min_element(load.begin(), load.end()) - load.begin());
        load[b] += cost[r];
        for (const GemmTile& t : rows[r]) seq[b].push_back(t);
    }
    size_t L = 0;
    for (const auto& q : seq) L = std::max(L, q.size());
    std::vector<GemmTile> out(L * G, GemmTile{-1, 0, 0});
    for (int b = 0; b < G; ++b)
        for (size_t k = 0; k < seq[b].size(); ++k) out[k * G + b] = seq[b][k];
    return out;
}

cudaError_t run_gemm(qg_plan* p, const GemmArgs& g, cudaStream_t s) {
    const int nt = pass_xin(g.pass) ? p->n_gx : p->n_gy;
    return timed(p, QG_K_GEMM, s, [&] {
        if (p->opts.dst_precision == QG_DST_FP32) return launch_gemm_simt(g, nt, s, use_pdl(p));
        PersistArgs a = p->pa;
        a.g4_accumulate = g.accumulate;
        const int grid = std::max(1, std::min(nt, p->n_sm));
        return launch_gemm_mt(a, g.pass, grid, p->opts.dst_precision, s, use_pdl(p));
    });
}

// psi_hat (XC) from the modal operand already in XA (and XQ for refinement).
cudaError_t run_dst_solve(qg_plan* p, cudaStream_t s) {
    const int f = p->op_fmt;
    cudaError_t e;
    // the last pass writes FP32 psi_hat; intermediate planes use the operand format
    if ((e = run_gemm(p, gemm_args(p, G1_FWD_X, p->XA, p->YA, f, f, 0), s))) return e;
    if ((e = run_gemm(p, gemm_args(p, G2_FWD_Y, p->YA, p->XB, f, f, 0), s))) return e;
    if ((e = run_gemm(p, gemm_args(p, G3_INV_X, p->XB, p->YB, f, f, 0), s))) return e;
    if ((e = run_gemm(p, gemm_args(p, G4_INV_Y, p->YB, p->XC, f, FMT_F32, 0), s))) return e;
    for (int r = 0; r < p->opts.refine_sweeps; ++r) {
        e = timed(p, QG_K_OTHER, s, [&] {
            return launch_residual(p->md, p->st_tiles, p->n_st, p->st_large, p->XQ, p->XC, p->XA, f, p->xplane, s,
                                   use_pdl(p));
        });
        if (e) return e;
        if ((e = run_gemm(p, gemm_args(p, G1_FWD_X, p->XA, p->YA, f, f, 0), s))) return e;
        if ((e = run_gemm(p, gemm_args(p, G2_FWD_Y, p->YA, p->XB, f, f, 0), s))) return e;
        if ((e = run_gemm(p, gemm_args(p, G3_INV_X, p->XB, p->YB, f, f, 0), s))) return e;
        if ((e = run_gemm(p, gemm_args(p, G4_INV_Y, p->YB, p->XC, f, FMT_F32, 1), s))) return e;
    }
    return cudaSuccess;
}

VjpArgs vjp_args(qg_plan* p) {
    VjpArgs v{};
    v.members = p->md;
    v.tiles = p->st_tiles;
    v.ntiles = p->n_st;
    v.tile_x = p->st_large ? kTileLX : kTileSX;
    v.tile_y = p->st_large ? kTileLY : kTileSY;
    v.max_nl = p->max_nl;
    v.n_members = p->n_members;
    v.pacc = p->vjp_acc;
    v.xa = p->XA;
    v.xa_fmt = p->op_fmt;
    v.xq = p->XQ;
    v.xplane = p->xplane;
    return v;
}

// psi_hat (XC) with the masked members' capacitance correction: solve, sigma at B into the
// operand, solve again (the operand is otherwise unchanged: it is zero on land).  With
// refinement the correction repeats once more, so that psi on B falls to the solve's
// precision squared (the FP64 capacitance matrices are exact, the solves are not).
cudaError_t run_inversion(qg_plan* p, cudaStream_t s) {
    cudaError_t e = run_dst_solve(p, s);
    if (e || p->n_cap == 0) return e;
    for (int c = 0; c < 1 + p->opts.refine_sweeps && !e; ++c) {
        e = timed(p, QG_K_OTHER, s, [&] {
            return launch_capacitance(p->md, p->cap_items, p->n_cap, p->XC, p->XA, p->op_fmt, p->XQ, p->xplane,
                                      p->cap_smem, s);
        });
        // a refinement sweep leaves its residual in the operand: rebuild it from the FP32
        // right-hand side (which holds the sources on B)
        if (!e && p->opts.refine_sweeps > 0)
            e = timed(p, QG_K_PREP, s, [&] {
                VjpArgs v = vjp_args(p);
                v.rhs = p->XQ;
                v.xq = nullptr;
                return launch_vjp_operand(v, nullptr, s);
            });
        if (!e) e = run_dst_solve(p, s);
    }
    return e;
}

// q (caller packing) -> optional internal copy + the modal GEMM operand.
cudaError_t run_prep(qg_plan* p, const float* q, float* copy, int zero_ring_copy, int bc_operand,
                     cudaStream_t s) {
    PrepArgs a{};
    a.members = p->md;
    a.tiles = p->st_tiles;
    a.q = q;
    a.copy = copy;
    a.zero_ring_copy = zero_ring_copy;
    a.bc_operand = bc_operand;
    a.xa = p->XA;
    a.xa_fmt = p->op_fmt;
    a.xq = p->XQ;
    a.xplane = p->xplane;
    a.tile_x = p->st_large ? kTileLX : kTileSX;
    a.tile_y = p->st_large ? kTileLY : kTileSY;
    return timed(p, QG_K_PREP, s, [&] { return launch_prep(a, p->n_st, s, use_pdl(p)); });
}

StencilArgs stencil_args(qg_plan* p, const float* params) {
    StencilArgs a{};
    a.members = p->md;
    a.tiles = p->st_tiles;
    a.maps = p->st_maps;
    a.params = params;
    a.xplane = p->xplane;
    a.xa_fmt = p->op_fmt;
    a.flags = p->flags;
    return a;
}

constexpr int kSweepRows[3] = {16, 32, 64};  // strip heights of sweep list v: kSweepRows[v % 3]
constexpr int kNumBN = 5;
constexpr int kGemmBN[kNumBN] = {144, 80, 48, 32, 16};  // tensor-core output tile widths the autotuner tries

// The multi-launch path's stencil launch: the column sweep if selected, else the tiles.
cudaError_t launch_stencil(qg_plan* p, StencilArgs a, cudaStream_t s, bool pdl) {
    const float* planes[3] = {p->S0, p->S1, p->S2};
    a.qin = planes[a.q_sel];
    a.psi_hat = p->XC;
    if (p->sw_sel >= 0) {
        const int v = p->sw_sel;
        const SweepItem* items[kSweepGroups];
        for (int k = 0; k < kSweepGroups; ++k) items[k] = p->sw_items_v[v] + p->sw_off[v][k];
        if (v >= 3) {
            int groups[kSweepGroups], n = 0;
            for (int g = 0; g < kSweepGroups; ++g)
                if (p->sw_cnt[v][g] > 0) groups[n++] = g;
            if (n <= 1 || !p->fork_ev || !p->fork_on)
                return launch_lsweep(a, items, p->sw_cnt[v], kSweepRows[v % 3], p->sw_grid, s, pdl);
            // fork: the first group on the stage's stream (after the last DST pass, with
            // programmatic dependent launch), the others on side streams after an event; join
            // them all back before the stage's next launch
            cudaError_t e = cudaEventRecord(p->fork_ev, s);
            for (int i = 0; i < n && !e; ++i) {
                const int g = groups[i];
                cudaStream_t ss = i == 0 ? s : p->side[(i - 1) % qg_plan::kSide];
                if (i > 0) e = cudaStreamWaitEvent(ss, p->fork_ev, 0);
                if (!e)
                    e = launch_lsweep_group(a, items[g], p->sw_cnt[v][g], kSweepRows[v % 3], p->sw_grid[g], g, ss,
                                            i == 0 && pdl);
                if (!e && i > 0) e = cudaEventRecord(p->join_ev[i], ss);
            }
            for (int i = 1; i < n && !e; ++i) e = cudaStreamWaitEvent(s, p->join_ev[i], 0);
            return e;
        }
        // the one-layer-per-lane sweep: class 0 of each layer count
        const SweepItem* it1[kMaxLayers];
        int cnt1[kMaxLayers], grid1[kMaxLayers];
        for (int k = 0; k < kMaxLayers; ++k) {
            it1[k] = items[k * kLSweepClasses];
            cnt1[k] = p->sw_cnt[v][k * kLSweepClasses];
            grid1[k] = p->sw_grid[k * kLSweepClasses];
        }
        return launch_sweep(a, it1, cnt1, kSweepRows[v], grid1, s, pdl);
    }
    return launch_stencil_mt(a, p->n_st, p->st_grid, p->max_nl, p->st_large, s, pdl);
}

struct Stage {
    float a, b;
};

int scheme_stages(int scheme, Stage* st) {
    switch (scheme) {
        case QG_SCHEME_HEUN:
            st[0] = {0.f, 1.f};
            st[1] = {0.5f, 0.5f};
            return 2;
        case QG_SCHEME_SSPRK3:
            st[0] = {0.f, 1.f};
            st[1] = {0.75f, 0.25f};
            st[2] = {1.f / 3.f, 2.f / 3.f};
            return 3;
        default:
            return 0;
    }
}

// Butcher tableaus of the schemes stepped in Butcher form: Euler and Tsit5 (Tsitouras 2011,
// the coefficients diffrax.Tsit5 uses).  a[s][j] (j < s) and b[s].
const Tableau* butcher(int scheme) {
    static const Tableau euler = {1, {{0}}, {1.0}};
    static const Tableau tsit5 = {
        6,
        {{0, 0, 0, 0, 0, 0},
         {0.161, 0, 0, 0, 0, 0},
         {-0.008480655492356989, 0.335480655492357, 0, 0, 0, 0},
         {2.897153057105493, -6.359448489975075, 4.3622954328695815, 0, 0, 0},
         {5.325864828439257, -11.748883564062828, 7.4955393428898365, -0.09249506636175525, 0, 0},
         {5.86145544294642, -12.92096931784711, 8.159367898576159, -0.071584973281401, -0.028269050394068383, 0}},
        {0.09646076681806523, 0.01, 0.4798896504144996, 1.379008574103742, -3.290069515436081, 2.324710524099774}};
    if (scheme == QG_SCHEME_EULER) return &euler;
    if (scheme == QG_SCHEME_TSIT5) return &tsit5;
    return nullptr;
}

// One Butcher-form step of the state in S0 (XA holding Cl2m BC(S0)): per stage the DST solve,
// the stencil in rhs mode writing k_s, and the combine into the next stage input (S1) or, at
// the last stage, the new state (S0) with the next step's operand.
cudaError_t run_one_step_butcher(qg_plan* p, const float* params, float dt, const Tableau& tb, cudaStream_t s) {
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < tb.n && !e; ++k) {
        if ((e = run_inversion(p, s))) break;
        StencilArgs a = stencil_args(p, params);
        a.q_sel = k == 0 ? 0 : 1;
        a.apply_bc = 1;
        a.dq = p->K + (size_t)k * p->state_size;
        e = timed(p, QG_K_STENCIL, s, [&] { return launch_stencil(p, a, s, use_pdl(p)); });
        if (e) break;
        RkCombineArgs c{};
        c.members = p->md;
        c.tiles = p->st_tiles;
        c.tile_x = p->st_large ? kTileLX : kTileSX;
        c.tile_y = p->st_large ? kTileLY : kTileSY;
        c.y0 = p->S0;
        c.k = p->K;
        c.kplane = p->state_size;
        const bool fin = k == tb.n - 1;
        c.n_k = k + 1;
        for (int j = 0; j <= k; ++j) c.coef[j] = (float)(fin ? tb.b[j] : tb.a[k + 1][j]);
        c.dt = dt;
        c.out = fin ? p->S0 : p->S1;
        c.xa = p->XA;
        c.xa_fmt = p->op_fmt;
        c.xq = p->XQ;
        c.xplane = p->xplane;
        e = timed(p, QG_K_OTHER, s, [&] { return launch_rk_combine(c, p->n_st, s, use_pdl(p)); });
    }
    return e;
}

// One time step of the state in S0 (XA holding Cl2m BC(S0)).  Stage k reads stage plane k
// (S0, S1, S2) and writes stage plane k + 1; the final stage updates S0 in place (it reads S0
// only pointwise there) and leaves XA ready for the next step.
cudaError_t run_one_step(qg_plan* p, const float* params, float dt, int scheme, cudaStream_t s) {
    if (const Tableau* tb = butcher(scheme)) return run_one_step_butcher(p, params, dt, *tb, s);
    Stage st[4];
    const int ns = scheme_stages(scheme, st);
    float* stage_buf[3] = {p->S0, p->S1, p->S2};
    cudaError_t e;
    for (int k = 0; k < ns; ++k) {
        if ((e = run_inversion(p, s))) return e;
        StencilArgs a = stencil_args(p, params);
        a.q_sel = k;
        a.apply_bc = 1;
        a.y0 = p->S0;
        const bool fin = (k == ns - 1);
        a.final_stage = fin;
        a.y_next = fin ? p->S0 : stage_buf[k + 1];
        a.a = st[k].a;
        a.b = st[k].b;
        a.dt = dt;
        a.xa = p->XA;
        a.xq = p->XQ;
        e = timed(p, QG_K_STENCIL, s, [&] { return launch_stencil(p, a, s, use_pdl(p)); });
        if (e) return e;
    }
    return cudaSuccess;
}

int cuda_err(cudaError_t e) { return e == cudaSuccess ? QG_OK : QG_ERR_CUDA; }

void select_sweep(qg_plan* p, int v) {
    p->sw_sel = v;
    if (v < 0) return;
    for (int g = 0; g < kSweepGroups; ++g) {
        const int k = g / kLSweepClasses, c = g % kLSweepClasses;
        // strips per CTA: one per warp (one-layer-per-lane sweep) or one per group of k + 1
        // warps (layer-per-warp sweep)
        const int per_cta = v >= 3 ? lsweep_strips_per_block(k + 1) : sweep_warps_per_block();
        const int per_sm = v >= 3 ? lsweep_blocks_per_sm(k + 1, c) : sweep_blocks_per_sm(k + 1);
        const int ctas = (p->sw_cnt[v][g] + per_cta - 1) / per_cta;
        p->sw_grid[g] = std::max(1, std::min(ctas, per_sm * std::max(p->n_sm, 1)));
    }
}

// Make stencil tile shape `large` the active one (tile list, TMA maps, launch grid).
void select_tile(qg_plan* p, int large) {
    p->st_large = large;
    p->st_tiles = p->st_tiles_v[large];
    p->n_st = p->n_st_v[large];
    p->st_maps = p->st_maps_v[large];
    const int bps = stencil_mt_blocks_per_sm(p->max_nl, large);
    p->st_grid = std::max(1, std::min(p->n_st, bps * std::max(p->n_sm, 1)));
    PersistArgs& a = p->pa;
    a.st = p->st_tiles;
    a.n_st = p->n_st;
    a.st_maps = p->st_maps;
    a.st_large = large;
    if (p->opts.dst_precision != QG_DST_FP32) persistent_smem_bytes(p->opts.dst_precision, p->max_nl, large, &a);
}

// Make tensor-core tile width kGemmBN[v] the active one (tile lists, persistent arguments).
void select_gemm(qg_plan* p, int v) {
    p->bn_sel = v;
    p->gx_tiles = p->gx_v[v];
    p->gy_tiles = p->gy_v[v];
    p->n_gx = p->n_gx_v[v];
    p->n_gy = p->n_gy_v[v];
    PersistArgs& a = p->pa;
    a.gx = p->gx_tiles;
    a.gy = p->gy_tiles;
    a.n_gx = p->n_gx;
    a.n_gy = p->n_gy;
    a.tile_n = kGemmBN[v];
}

// Autotuner: time the four DST passes with each tensor-core tile width (zero planes) and keep
// the fastest.
cudaError_t autotune_gemm(qg_plan* p) {
    cudaStream_t s = p->cap;
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (!e) e = cudaEventCreate(&e1);
    if (e) return e;
    int best = 0;
    for (int v = 0; v < p->n_bn && !e; ++v) {
        select_gemm(p, v);
        float ms = 0.f;
        e = run_dst_solve(p, s);
        if (!e) e = cudaEventRecord(e0, s);
        for (int rep = 0; rep < 3 && !e; ++rep) e = run_dst_solve(p, s);
        if (!e) e = cudaEventRecord(e1, s);
        if (!e) e = cudaEventSynchronize(e1);
        if (!e) e = cudaEventElapsedTime(&ms, e0, e1);
        p->tune_gemm_ms[v] = ms / 3.f;
        if (!e && p->tune_gemm_ms[v] < p->tune_gemm_ms[best]) best = v;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (!e) select_gemm(p, best);
    return e;
}

int autotune_engine(qg_plan* p);

// Autotuner: time every stencil variant (tile shapes, sweep strip heights) in its setting,
// one RK stage (the four DST passes, then the step-mode stencil) on the plan's own planes
// (zero state, zero parameters), with CUDA events; the passes are common to all variants,
// so the differences are the stencil's, including what the GEMM passes leave in L2.  The
// fastest tile shape is the persistent kernel's; the fastest variant overall is the
// multi-launch path's.
cudaError_t autotune_stencil(qg_plan* p) {
    cudaStream_t s = p->cap;
    cudaEvent_t e0, e1;
    cudaError_t e = cudaEventCreate(&e0);
    if (!e) e = cudaEventCreate(&e1);
    if (e) return e;
    // every parameter non-zero while timing, so that every term (the biharmonic's lap(q) pass
    // included) runs as it will in the integration
    {
        std::vector<float> ones((size_t)p->n_members * QG_NPARAMS, 1.f);
        e = cudaMemcpy(p->params, ones.data(), ones.size() * sizeof(float), cudaMemcpyHostToDevice);
        if (e) return e;
    }
    const int tile_default = p->st_large;
    for (int v = 0; v < QG_STENCIL_VARIANTS && !e; ++v) {
        if (v < 2) {
            select_tile(p, v);
            select_sweep(p, -1);
        } else {
            select_tile(p, tile_default);
            select_sweep(p, v - 2);
        }
        StencilArgs a = stencil_args(p, p->params);
        a.q_sel = 1;
        a.apply_bc = 1;
        a.y0 = p->S0;
        a.y_next = p->S2;
        a.a = 0.5f;
        a.b = 0.5f;
        a.dt = 1.f;
        a.xa = p->XA;
        float ms = 0.f;
        for (int rep = 0; rep < 1 && !e; ++rep) {
            e = run_dst_solve(p, s);
            if (!e) e = launch_stencil(p, a, s, false);
        }
        if (!e) e = cudaEventRecord(e0, s);
        for (int rep = 0; rep < 3 && !e; ++rep) {
            e = run_dst_solve(p, s);
            if (!e) e = launch_stencil(p, a, s, false);
        }
        if (!e) e = cudaEventRecord(e1, s);
        if (!e) e = cudaEventSynchronize(e1);
        if (!e) e = cudaEventElapsedTime(&ms, e0, e1);
        p->tune_ms[v] = ms / 3.f;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (e) return e;
    const int tile = p->tune_ms[1] < p->tune_ms[0] ? 1 : 0;
    int best = tile;
    for (int v = 2; v < QG_STENCIL_VARIANTS; ++v)
        if (p->tune_ms[v] < p->tune_ms[best]) best = v;
    select_tile(p, tile);
    select_sweep(p, best >= 2 ? best - 2 : -1);
    e = cudaMemsetAsync(p->S2, 0, sizeof(float) * p->xplane, s);
    if (!e) e = cudaMemsetAsync(p->params, 0, sizeof(float) * p->n_members * QG_NPARAMS, s);
    if (!e) e = cudaMemsetAsync(p->XA, 0, sizeof(float) * p->xplane, s);
    if (!e) e = cudaStreamSynchronize(s);
    return e;
}

}  // namespace

namespace qg {
cudaError_t tmap_encode(void* map, int bf16, int rank, const void* base, const uint64_t* dims,
                        const uint64_t* strides_bytes, const uint32_t* box, int swizzle128) {
    if (!g_encode || rank < 1 || rank > 5) return cudaErrorInvalidValue;
    const int es = bf16 ? 2 : 4;
    if (((uintptr_t)base & 15) || (box[0] * es) % 16) return cudaErrorInvalidValue;
    cuuint64_t d[5];
    cuuint64_t st[4];
    cuuint32_t b[5], e[5];
    for (int k = 0; k < rank; ++k) {
        d[k] = dims[k];
        b[k] = box[k];
        e[k] = 1;
        if (k < rank - 1) {
            st[k] = strides_bytes[k];
            if (st[k] % 16) return cudaErrorInvalidValue;
        }
    }
    CUresult r = g_encode(static_cast<CUtensorMap*>(map),
                          bf16 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, rank,
                          const_cast<void*>(base), d, st, b, e, CU_TENSOR_MAP_INTERLEAVE_NONE,
                          swizzle128 ? CU_TENSOR_MAP_SWIZZLE_128B : CU_TENSOR_MAP_SWIZZLE_NONE,
                          CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}
}  // namespace qg

// =======================================================================================
// C ABI
// =======================================================================================
extern "C" {

const char* qg_strerror(int code) {
    if (code < 0 || code >= (int)(sizeof(kErrStr) / sizeof(kErrStr[0]))) return "unknown error";
    return kErrStr[code];
}

int qg_plan_create(const qg_member_desc* members, int n_members, const qg_options* opts,
                   qg_plan** out) {
    if (!members || !out) return QG_ERR_NULL;
    *out = nullptr;
    if (n_members < 1) return QG_ERR_SHAPE;
    qg_options o{};
    o.dst_precision = QG_DST_FP32;
    o.refine_sweeps = 0;
    o.use_graphs = 1;
    o.persistent = 1;
    o.autotune = 1;
    if (opts) o = *opts;
    if (o.dst_precision < QG_DST_FP32 || o.dst_precision > QG_DST_BF16X3) return QG_ERR_ARG;
    if (o.refine_sweeps < 0 || o.refine_sweeps > 1) return QG_ERR_ARG;
    if (o.cluster < 0 || o.cluster > 2) return QG_ERR_ARG;
    if (o.stencil < 0 || o.stencil > QG_STENCIL_VARIANTS) return QG_ERR_ARG;
    if (o.gemm_tile != 0 && std::find(kGemmBN, kGemmBN + kNumBN, o.gemm_tile) == kGemmBN + kNumBN)
        return QG_ERR_ARG;
    for (int i = 0; i < n_members; ++i) {
        const int v = validate_member(members[i]);
        if (v != QG_OK) return v;
    }
    qg_plan* p = new (std::nothrow) qg_plan();
    if (!p) return QG_ERR_CUDA;
    p->n_members = n_members;
    p->opts = o;
    p->desc.assign(members, members + n_members);
    cudaGetDevice(&p->device);
    if (tmap_init() != cudaSuccess || persistent_init() != cudaSuccess) {
        delete p;
        return QG_ERR_UNSUPPORTED;
    }
    if (o.dst_precision != QG_DST_FP32) {
        if (gemm_tc_init() != cudaSuccess) {
            delete p;
            return QG_ERR_UNSUPPORTED;
        }
        p->op_fmt = (o.dst_precision == QG_DST_BF16X3) ? FMT_BF16X2 : FMT_F32;
    }
    cudaError_t e = cudaDeviceGetAttribute(&p->n_sm, cudaDevAttrMultiProcessorCount, p->device);
    {
        // default stencil tile shape (the autotuner may overrule it): the large tile once it
        // still gives every SM two tiles per stage
        int64_t large_tiles = 0;
        for (int i = 0; i < n_members; ++i)
            large_tiles += (int64_t)((members[i].ny + 2 + kTileLY - 1) / kTileLY) *
                           ((members[i].nx + 2 + kTileLX - 1) / kTileLX);
        p->st_large = large_tiles >= 2 * (int64_t)std::max(p->n_sm, 1);
    }
    std::vector<StencilTile> st_v[2];
    std::vector<SweepItem> sw_v[kSweepLists];
    std::vector<CapItem> cap;
    bool too_large = false;
    // geometry and offsets
    p->mh.resize(n_members);
    int64_t off_state = 0, off_x = 0, off_y = 0, off_layer = 0;
    std::vector<StencilTile> st;
    const bool tc = o.dst_precision != QG_DST_FP32;
    const int BMg = tc ? 128 : kSimtBM;
    const int n_bn = tc ? kNumBN : 1;
    std::vector<GemmTile> gxv[kNumBN], gyv[kNumBN];
    std::map<long long, std::pair<float*, uint16_t*>> dst_cache;  // (size, pitch) -> device DST-I matrix
    for (int i = 0; i < n_members; ++i) {
        const qg_member_desc& d = members[i];
        MemberDev& M = p->mh[i];
        double Cl2m[64], Cm2l[64], lam[8];
        member_constants(d, M, Cl2m, Cm2l, lam);
        const int n = d.n_layers;
        const double dx = d.Lx / d.nx, dy = d.Ly / d.ny;
        p->desc[i].has_modes = 1;  // remember what the plan uses
        for (int k = 0; k < n * n; ++k) {
            p->desc[i].Cl2m[k] = Cl2m[k];
            p->desc[i].Cm2l[k] = Cm2l[k];
        }
        for (int k = 0; k < n; ++k) p->desc[i].lambdas[k] = lam[k];
        M.off_state = off_state;
        M.off_x = off_x;
        M.off_y = off_y;
        M.off_layer = off_layer;
        p->member_off.push_back(off_state);
        off_state += (int64_t)n * M.Ny * M.Nx;
        off_x += (int64_t)n * M.Ny * M.Px;
        off_y += (int64_t)n * M.Nx * M.Py;
        off_layer += n;
        p->max_nl = std::max(p->max_nl, n);
        // constant fields
        std::vector<float> by(M.Ny), F(M.Ny), ex, ey;
        for (int j = 0; j < M.Ny; ++j) {
            const double y = j * dy;
            by[j] = (float)(d.beta * (y - d.Ly / 2.0));
            F[j] = (float)(d.wind_profile == QG_WIND_SINGLE ? std::sin(M_PI * y / d.Ly)
                                                             : -std::sin(2.0 * M_PI * y / d.Ly));
        }
        dst_eigs(M.Nx, dx, ex);
        dst_eigs(M.Ny, dy, ey);
        float *dby, *dF, *dex, *dey;
        if ((e = upload(p, &dby, by)) || (e = upload(p, &dF, F)) || (e = upload(p, &dex, ex)) ||
            (e = upload(p, &dey, ey)))
            break;
        M.by = dby;
        M.F = dF;
        M.ex = dex;
        M.ey = dey;
        {
            // bf16 hi/lo split of a DST matrix (hi plane then lo plane)
            auto split = [&](const std::vector<float>& S, uint16_t** dst) {
                std::vector<uint16_t> h(2 * S.size());
                for (size_t k = 0; k < S.size(); ++k) {
                    auto bf = [](float f) {
                        uint32_t u;
                        std::memcpy(&u, &f, 4);
                        u += 0x7fffu + ((u >> 16) & 1u);  // round to nearest even
                        return (uint16_t)(u >> 16);
                    };
                    const uint16_t hi = bf(S[k]);
                    uint32_t hu = (uint32_t)hi << 16;
                    float hf;
                    std::memcpy(&hf, &hu, 4);
                    h[k] = hi;
                    h[S.size() + k] = bf(S[k] - hf);
                }
                return upload(p, dst, h);
            };
            // The DST-I matrix of a size and pitch is the same for every member: one device copy
            // per (size, pitch), shared, so that every GEMM pass reads it from L2 instead of one
            // DRAM copy per member (28 MB per pass on the 256-member ensemble).
            auto shared_dst = [&](int nn, int ld, float** f32, uint16_t** bf) -> cudaError_t {
                const long long key = (long long)nn << 32 | (unsigned)ld;
                auto it = dst_cache.find(key);
                if (it == dst_cache.end()) {
                    std::vector<float> S;
                    dst_matrix(nn, ld, S);
                    float* d32 = nullptr;
                    uint16_t* dbf = nullptr;
                    cudaError_t ee = upload(p, &d32, S);
                    if (!ee && o.dst_precision == QG_DST_BF16X3) ee = split(S, &dbf);
                    if (ee) return ee;
                    it = dst_cache.emplace(key, std::make_pair(d32, dbf)).first;
                }
                *f32 = it->second.first;
                *bf = it->second.second;
                return cudaSuccess;
            };
            float *dSx, *dSy;
            uint16_t *bx, *byy;
            if ((e = shared_dst(M.Nx, M.Px, &dSx, &bx)) || (e = shared_dst(M.Ny, M.Py, &dSy, &byy))) break;
            M.Sx = dSx;
            M.Sy = dSy;
            M.Sx_bf = bx;
            M.Sy_bf = byy;
        }
        // masked basin: land mask, boundary points and inverse capacitance matrices
        if (d.mask) {
            std::vector<uint8_t> mk(d.mask, d.mask + (size_t)M.Ny * M.Nx);
            uint8_t* dm;
            if ((e = upload(p, &dm, mk))) break;
            M.mask = dm;
            const std::vector<int> B = land_boundary(d);
            if ((int)B.size() > kMaxBoundary) {
                e = cudaErrorInvalidValue;
                too_large = true;
                break;
            }
            if (!B.empty()) {
                std::vector<double> cinv;
                if (!capacitance_inverse(d, lam, n, B, cinv)) {
                    e = cudaErrorInvalidValue;
                    break;
                }
                int* db;
                double* dc;
                if ((e = upload(p, &db, B)) || (e = upload(p, &dc, cinv))) break;
                M.nb = (int)B.size();
                M.bidx = db;
                M.cinv = dc;
                for (int m = 0; m < n; ++m)
                    for (int r0 = 0; r0 < M.nb; r0 += kCapRows) cap.push_back({i, m, r0});
                p->cap_smem = std::max(p->cap_smem, (size_t)M.nb * sizeof(double));
            }
        }
        // column-sweep strips
        for (int v = 0; v < kSweepLists; ++v) {
            const int R = kSweepRows[v % 3], W = v >= 3 ? lsweep_columns() : sweep_columns();
            const int bands = v >= 3 ? lsweep_bands(M.Ny, R) : (M.Ny + R - 1) / R;
            for (int sy = 0; sy < bands; ++sy)
                for (int sx = 0; sx < (M.Nx + W - 1) / W; ++sx) sw_v[v].push_back({i, sx, sy});
        }
        // tiles
        for (int v = 0; v < 2; ++v) {
            const int TX = v ? kTileLX : kTileSX, TY = v ? kTileLY : kTileSY;
            for (int ty = 0; ty < (M.Ny + TY - 1) / TY; ++ty)
                for (int tx = 0; tx < (M.Nx + TX - 1) / TX; ++tx) st_v[v].push_back({i, ty, tx});
        }
        for (int v = 0; v < n_bn; ++v) {
            const int BNg = tc ? kGemmBN[v] : kSimtBN;
            for (int mt = 0; mt < (n * M.Ny + BMg - 1) / BMg; ++mt)
                for (int nt = 0; nt < (M.Nx + BNg - 1) / BNg; ++nt) gxv[v].push_back({i, mt, nt});
            for (int mt = 0; mt < (n * M.Nx + BMg - 1) / BMg; ++mt)
                for (int nt = 0; nt < (M.Ny + BNg - 1) / BNg; ++nt) gyv[v].push_back({i, mt, nt});
        }
    }
    if (e == cudaSuccess) {
        p->state_size = off_state;
        p->xplane = off_x;
        p->yplane = off_y;
        p->total_layers = off_layer;
        std::vector<MemberDev> mv(p->mh);
        e = upload(p, &p->md, mv);
    }
    if (e == cudaSuccess) {
        p->n_bn = n_bn;
        for (int v = 0; v < 2 && !e; ++v) {
            p->n_st_v[v] = (int)st_v[v].size();
            e = upload(p, &p->st_tiles_v[v], st_v[v]);
        }
        if (!e && !cap.empty()) {
            p->n_cap = (int)cap.size();
            e = upload(p, &p->cap_items, cap);
            if (!e) e = capacitance_init(p->cap_smem);
        }
        for (int v = 0; v < kSweepLists && !e; ++v) {
            // group by layer count and strip class: one sweep launch per group
            std::vector<SweepItem> g;
            for (int k = 0; k < kSweepGroups; ++k) {
                p->sw_off[v][k] = (int)g.size();
                for (const SweepItem& it : sw_v[v]) {
                    const qg_member_desc& d = members[it.member];
                    const int cls = v >= 3 ? lsweep_item_class(d.ny + 2, d.nx + 2, d.mask != nullptr, it.sx, it.sy,
                                                               kSweepRows[v % 3])
                                           : 0;
                    if (d.n_layers * kLSweepClasses + cls == k + kLSweepClasses) g.push_back(it);
                }
                p->sw_cnt[v][k] = (int)g.size() - p->sw_off[v][k];
            }
            p->n_sw_v[v] = (int)g.size();
            e = upload(p, &p->sw_items_v[v], g);
        }
        if (tc) {
            std::vector<int> kx(n_members), ky(n_members);  // contraction lengths of the x / y passes
            for (int i = 0; i < n_members; ++i) {
                kx[i] = members[i].nx + 2;
                ky[i] = members[i].ny + 2;
            }
            for (int v = 0; v < n_bn; ++v) {
                gxv[v] = schedule_tiles(gxv[v], p->n_sm, kx);
                gyv[v] = schedule_tiles(gyv[v], p->n_sm, ky);
            }
        }
        for (int v = 0; v < n_bn && !e; ++v) {
            p->n_gx_v[v] = (int)gxv[v].size();
            p->n_gy_v[v] = (int)gyv[v].size();
            if (!(e = upload(p, &p->gx_v[v], gxv[v]))) e = upload(p, &p->gy_v[v], gyv[v]);
        }
        if (!e) {
            p->gx_tiles = p->gx_v[0];
            p->gy_tiles = p->gy_v[0];
            p->n_gx = p->n_gx_v[0];
            p->n_gy = p->n_gy_v[0];
        }
    }
    if (e == cudaSuccess) {
        const size_t xb = (size_t)p->xplane * 4, yb = (size_t)p->yplane * 4;
        if (!(e = dalloc(p, &p->XA, xb)) && !(e = dalloc(p, &p->XB, xb)) && !(e = dalloc(p, &p->XC, xb)) &&
            !(e = dalloc(p, &p->YA, yb)) && !(e = dalloc(p, &p->YB, yb)) && !(e = dalloc(p, &p->S0, xb)) &&
            !(e = dalloc(p, &p->S1, xb)) &&
            !(e = dalloc(p, &p->S2, xb)) && !(e = dalloc(p, &p->params, (size_t)n_members * QG_NPARAMS * 4)) &&
            !(e = dalloc(p, &p->flags, 16)) && !(e = dalloc(p, &p->bar, 16)))
            e = dalloc(p, &p->diag_acc, (size_t)2 * p->total_layers * sizeof(double));
        if (!e) e = dalloc(p, &p->vjp_acc, (size_t)n_members * QG_NPARAMS * sizeof(double));
        if (!e) e = dalloc(p, (uint8_t**)&p->stats_acc, 64);
        if (!e && o.refine_sweeps > 0) e = dalloc(p, &p->XQ, xb);
        if (!e) e = dalloc(p, &p->K, (size_t)6 * p->state_size * sizeof(float));  // Tsit5: 6 stages
    }
    if (e == cudaSuccess && tc) {
        // one set of TMA descriptors per (member, pass); the planes never move
        std::vector<uint8_t> maps((size_t)n_members * 4 * kTcMapsBytes);
        const void* in_plane[4] = {p->XA, p->YA, p->XB, p->YB};
        const int64_t in_elems[4] = {p->xplane, p->yplane, p->xplane, p->yplane};
        for (int i = 0; i < n_members && !e; ++i)
            for (int pass = 0; pass < 4 && !e; ++pass)
                e = gemm_tc_encode(p->mh[i], pass, in_plane[pass], in_elems[pass], o.dst_precision,
                                   maps.data() + ((size_t)i * 4 + pass) * kTcMapsBytes);
        if (!e) e = upload(p, (uint8_t**)&p->tc_maps, maps);
    }
    if (e == cudaSuccess) {
        // TMA descriptors of the stencil's halo boxes: the three stage planes and psi_hat
        const float* planes[4] = {p->S0, p->S1, p->S2, p->XC};
        for (int v = 0; v < 2 && !e; ++v) {
            std::vector<uint8_t> maps((size_t)n_members * kStencilMapsBytes);
            for (int i = 0; i < n_members && !e; ++i)
                e = stencil_encode_maps(p->mh[i], planes, v, maps.data() + (size_t)i * kStencilMapsBytes);
            if (!e) e = upload(p, (uint8_t**)&p->st_maps_v[v], maps);
        }
    }
    if (e == cudaSuccess) {
        PersistArgs& a = p->pa;
        a.members = p->md;
        a.gx = p->gx_tiles;
        a.gy = p->gy_tiles;
        a.n_gx = p->n_gx;
        a.n_gy = p->n_gy;
        a.tile_n = tc ? kGemmBN[0] : kSimtBN;
        a.max_nl = p->max_nl;
        a.tc_maps = p->tc_maps;
        a.XA = p->XA;
        a.YA = p->YA;
        a.YB = p->YB;
        a.XB = p->XB;
        a.XC = p->XC;
        a.S[0] = p->S0;
        a.S[1] = p->S1;
        a.S[2] = p->S2;
        a.params = p->params;
        a.xplane = p->xplane;
        a.yplane = p->yplane;
        a.op_fmt = p->op_fmt;
        a.flags = p->flags;
        a.bar_count = p->bar;
        a.bar_gen = p->bar + 1;
        a.bar_wait = kTimeoutCycles;
        select_tile(p, p->st_large);
        // side streams for the sweep's parallel branches, before the autotuner times them
        for (int i = 0; i < qg_plan::kSide && e == cudaSuccess; ++i)
            e = cudaStreamCreateWithFlags(&p->side[i], cudaStreamNonBlocking);
        for (int i = 0; i < kSweepGroups && e == cudaSuccess; ++i)
            e = cudaEventCreateWithFlags(&p->join_ev[i], cudaEventDisableTiming);
        // the fork event last: its presence switches the sweep's groups to parallel branches
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&p->fork_ev, cudaEventDisableTiming);
        // a forced choice (qg_options.gemm_tile / .stencil) skips that half of the autotuner
        if (!e && o.autotune && tc && !o.gemm_tile) e = autotune_gemm(p);
        if (!e && tc && o.gemm_tile)
            for (int v = 0; v < kNumBN; ++v)
                if (kGemmBN[v] == o.gemm_tile) select_gemm(p, v);
        if (!e && o.autotune && !o.stencil) e = autotune_stencil(p);
        if (!e && o.stencil > 0) {
            // a forced variant (tests, benchmarks of one variant)
            const int v = o.stencil - 1;
            if (v < 2) select_tile(p, v);
            select_sweep(p, v >= 2 ? v - 2 : -1);
        }
    }
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&p->cap, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    if (e == cudaSuccess && o.cluster != 2) {
        // cluster-resident stepping: every member alike in layers and grid, no land
        bool alike = true;
        for (int i = 0; i < n_members; ++i)
            alike = alike && !members[i].mask && members[i].n_layers == members[0].n_layers &&
                    members[i].nx == members[0].nx && members[i].ny == members[0].ny;
        if (alike) {
            p->cl_nl = members[0].n_layers;
            p->cl_C = cluster_size_for(p->cl_nl, members[0].ny + 2, members[0].nx + 2, &p->cl_smem);
        }
        if (p->cl_C > 0 && o.cluster == 1) p->cl_use = true;
        // the autotuner weighs it only when no stencil variant or tile width is forced (a
        // forced choice asks for the multi-launch path)
        if (p->cl_C > 0 && o.cluster == 0 && o.autotune && !o.stencil && !o.gemm_tile) {
            const int r = autotune_engine(p);
            if (r != QG_OK) e = cudaErrorUnknown;
        }
    }
    if (e != cudaSuccess) {
        qg_plan_destroy(p);
        return too_large ? QG_ERR_TOO_LARGE : QG_ERR_CUDA;
    }
    *out = p;
    return QG_OK;
}

void qg_plan_destroy(qg_plan* p) {
    if (!p) return;
    cudaDeviceSynchronize();
    if (p->graph.exec) cudaGraphExecDestroy(p->graph.exec);
    if (p->graph.exec_k) cudaGraphExecDestroy(p->graph.exec_k);
    if (p->vjp_graph.exec) cudaGraphExecDestroy(p->vjp_graph.exec);
    for (auto& v : p->ev)
        for (auto& pr : v) {
            cudaEventDestroy(pr.first);
            cudaEventDestroy(pr.second);
        }
    if (p->cap) cudaStreamDestroy(p->cap);
    for (cudaStream_t x : p->side)
        if (x) cudaStreamDestroy(x);
    if (p->fork_ev) cudaEventDestroy(p->fork_ev);
    for (cudaEvent_t x : p->join_ev)
        if (x) cudaEventDestroy(x);
    for (void* a : p->allocs) cudaFree(a);
    delete p;
}

int64_t qg_plan_state_size(const qg_plan* p) { return p ? p->state_size : -1; }

int64_t qg_plan_member_offset(const qg_plan* p, int m) {
    if (!p || m < 0 || m >= p->n_members) return -1;
    return p->member_off[m];
}

int qg_plan_member_modes(const qg_plan* p, int m, double* lambdas, double* Cl2m, double* Cm2l) {
    if (!p) return QG_ERR_NULL;
    if (m < 0 || m >= p->n_members) return QG_ERR_ARG;
    const qg_member_desc& d = p->desc[m];
    const int n = d.n_layers;
    if (lambdas) std::memcpy(lambdas, d.lambdas, sizeof(double) * n);
    if (Cl2m) std::memcpy(Cl2m, d.Cl2m, sizeof(double) * n * n);
    if (Cm2l) std::memcpy(Cm2l, d.Cm2l, sizeof(double) * n * n);
    return QG_OK;
}

int qg_invert(qg_plan* p, const float* q, float* psi, void* stream) {
    if (!p || !q || !psi) return QG_ERR_NULL;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = run_prep(p, q, nullptr, 0, 0, s);
    if (!e) e = run_inversion(p, s);
    if (!e)
        e = timed(p, QG_K_OTHER, s, [&] {
            return launch_mode_to_layer(p->md, p->st_tiles, p->n_st, p->st_large, p->XC, psi, s, use_pdl(p));
        });
    return cuda_err(e);
}

int qg_project(qg_plan* p, const float* h, const float* u, const float* v, float* h_g, float* u_g, float* v_g,
               float* psi, void* stream) {
    if (!p || !h || !u || !v || !h_g || !u_g || !v_g) return QG_ERR_NULL;
    if (p->n_cap > 0) return QG_ERR_UNSUPPORTED;
    for (const MemberDev& M : p->mh)
        if (M.barotropic) return QG_ERR_UNSUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
    // the PV and psi in two of the Butcher stage planes (caller packing)
    float* q = p->K;
    float* ps = psi ? psi : p->K + p->state_size;
    cudaError_t e = timed(p, QG_K_OTHER, s, [&] {
        return launch_project_q(p->md, p->st_tiles, p->n_st, p->st_large, h, u, v, q, s);
    });
    if (e) return cuda_err(e);
    const int r = qg_invert(p, q, ps, stream);
    if (r != QG_OK) return r;
    e = timed(p, QG_K_OTHER, s, [&] {
        return launch_project_g(p->md, p->st_tiles, p->n_st, p->st_large, ps, h_g, u_g, v_g, s);
    });
    return cuda_err(e);
}

int qg_project_vjp(qg_plan* p, const float* hg_bar, const float* ug_bar, const float* vg_bar, float* h_bar,
                   float* u_bar, float* v_bar, void* stream) {
    if (!p || !hg_bar || !ug_bar || !vg_bar || !h_bar || !u_bar || !v_bar) return QG_ERR_NULL;
    if (p->n_cap > 0) return QG_ERR_UNSUPPORTED;
    for (const MemberDev& M : p->mh)
        if (M.barotropic) return QG_ERR_UNSUPPORTED;
    cudaStream_t s = (cudaStream_t)stream;
    // psi_bar and q_bar in two Butcher stage planes the forward projection does not use
    float* psib = p->K + 2 * p->state_size;
    float* qb = p->K + 3 * p->state_size;
    cudaError_t e = timed(p, QG_K_OTHER, s, [&] {
        return launch_project_g_vjp(p->md, p->st_tiles, p->n_st, p->st_large, hg_bar, ug_bar, vg_bar, psib, s);
    });
    if (e) return cuda_err(e);
    const int r = qg_invert_vjp(p, psib, qb, stream);
    if (r != QG_OK) return r;
    e = timed(p, QG_K_OTHER, s, [&] {
        return launch_project_q_vjp(p->md, p->st_tiles, p->n_st, p->st_large, qb, h_bar, u_bar, v_bar, s);
    });
    return cuda_err(e);
}

namespace {
// dq = vector_field(q) (with the BC on read when bc), every member, on stream s.
cudaError_t rhs_core(qg_plan* p, const float* q, float* dq, const float* params, int bc, cudaStream_t s) {
    // q is staged into the S1 plane (TMA-able pitch); the stencil applies the BC on read
    cudaError_t e = run_prep(p, q, p->S1, 0, bc, s);
    if (!e) e = run_inversion(p, s);
    if (!e) {
        StencilArgs a = stencil_args(p, params);
        a.q_sel = 1;
        a.apply_bc = bc;
        a.dq = dq;
        e = timed(p, QG_K_STENCIL, s, [&] { return launch_stencil(p, a, s, use_pdl(p)); });
    }
    return e;
}
}  // namespace

int qg_rhs(qg_plan* p, const float* q, float* dq, const float* params, int flags, void* stream) {
    if (!p || !q || !dq || !params) return QG_ERR_NULL;
    if (flags & ~QG_RHS_APPLY_BC) return QG_ERR_ARG;
    return cuda_err(rhs_core(p, q, dq, params, (flags & QG_RHS_APPLY_BC) ? 1 : 0, (cudaStream_t)stream));
}

int qg_step(qg_plan* p, float* q, const float* params, double dt, int n_steps, int scheme,
            int flags, void* stream) {
    if (!p || !q || !params) return QG_ERR_NULL;
    if (n_steps < 0 || (flags & ~QG_STEP_APPLY_BC)) return QG_ERR_ARG;
    Stage st[4];
    if (scheme_stages(scheme, st) == 0 && !butcher(scheme)) return QG_ERR_ARG;
    if (!(dt == dt)) return QG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (p->cl_use && n_steps > 0 && !butcher(scheme)) {
        // one launch: every stage of every step, q and params read in the caller's packing
        const int ns = scheme_stages(scheme, st);
        float sa[4], sb[4];
        for (int k = 0; k < ns; ++k) {
            sa[k] = st[k].a;
            sb[k] = st[k].b;
        }
        const cudaError_t ec = timed(p, QG_K_PERSISTENT, s, [&] {
            return launch_cluster(p->md, p->n_members, p->cl_nl, p->cl_C, p->cl_smem, q, params,
                                  (flags & QG_STEP_APPLY_BC) ? 1 : 0, n_steps, ns, sa, sb, (float)dt, p->flags, s);
        });
        return cuda_err(ec);
    }
    cudaError_t e = cudaMemcpyAsync(p->params, params, sizeof(float) * p->n_members * QG_NPARAMS,
                                    cudaMemcpyDeviceToDevice, s);
    // the state lives in S0 for the whole call; its ring is zeroed only for a new
    // integration (integrate() applies the BC to state0), stage inputs always read a zero ring
    if (!e) e = run_prep(p, q, p->S0, (flags & QG_STEP_APPLY_BC) ? 1 : 0, 1, s);
    if (e) return cuda_err(e);
    // while profiling, the multi-launch path runs so that every kernel class gets its events
    const bool persistent = p->opts.persistent && p->opts.dst_precision != QG_DST_FP32 &&
                            p->opts.refine_sweeps == 0 && !p->profiling && p->n_cap == 0 && !butcher(scheme);
    const bool use_graph = p->opts.use_graphs && !p->profiling;
    if (persistent && n_steps > 0) {
        PersistArgs a = p->pa;
        a.n_stages = scheme_stages(scheme, st);
        for (int k = 0; k < a.n_stages; ++k) {
            a.sa[k] = st[k].a;
            a.sb[k] = st[k].b;
        }
        a.dt = (float)dt;
        a.n_steps = n_steps;
        a.g4_accumulate = 0;
        const int grid = std::max(1, std::min(p->n_sm, std::max(p->n_st, std::max(p->n_gx, p->n_gy))));
        // a launch that gave up at a grid barrier leaves arrivals behind: start from zero
        e = cudaMemsetAsync(p->bar, 0, 2 * sizeof(unsigned), s);
        if (!e)
            e = timed(p, QG_K_PERSISTENT, s, [&] { return launch_persistent(a, grid, p->opts.dst_precision, s); });
    } else if (!use_graph) {
        for (int k = 0; k < n_steps && !e; ++k) e = run_one_step(p, p->params, (float)dt, scheme, s);
    } else if (n_steps > 0) {
        StepGraph& g = p->graph;
        if (g.dt != dt || g.scheme != scheme) {
            for (cudaGraphExec_t* x : {&g.exec, &g.exec_k})
                if (*x) {
                    cudaGraphExecDestroy(*x);
                    *x = nullptr;
                }
            g.dt = dt;
            g.scheme = scheme;
        }
        // capture `steps` consecutive steps into *out
        auto capture = [&](int steps, cudaGraphExec_t* out) {
            cudaGraph_t graph = nullptr;
            cudaError_t ec = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
            if (!ec) {
                cudaError_t e1 = cudaSuccess;
                for (int k = 0; k < steps && !e1; ++k) e1 = run_one_step(p, p->params, (float)dt, scheme, p->cap);
                ec = cudaStreamEndCapture(p->cap, &graph);
                if (!ec) ec = e1;
            }
            if (!ec) ec = cudaGraphInstantiate(out, graph, 0);
            if (graph) cudaGraphDestroy(graph);
            if (ec) *out = nullptr;
            return ec;
        };
        int left = n_steps;
        if (left >= kGraphSteps && !g.exec_k) e = capture(kGraphSteps, &g.exec_k);
        for (; left >= kGraphSteps && !e; left -= kGraphSteps) e = cudaGraphLaunch(g.exec_k, s);
        if (!e && left > 0 && !g.exec) e = capture(1, &g.exec);
        for (; left > 0 && !e; --left) e = cudaGraphLaunch(g.exec, s);
        if (e) return cuda_err(e);
    }
    if (!e)
        e = timed(p, QG_K_OTHER, s, [&] {
            return launch_unpack(p->md, p->st_tiles, p->n_st, p->st_large, p->S0, q, s, use_pdl(p));
        });
    return cuda_err(e);
}

namespace {
// q_bar = (d dq / d q)^T dq_bar of the rhs at q; the parameter cotangents are added to the
// plan's FP64 accumulators (zeroed by the caller).  psi: the layer psi of q (caller packing)
// when the caller has it, else null (computed here).
cudaError_t rhs_vjp_core(qg_plan* p, const float* q, const float* params, const float* dq_bar, float* q_bar,
                         int bc, cudaStream_t s, const float* psi = nullptr) {
    cudaError_t e = cudaSuccess;
    if (!psi) {
        // forward psi (layer, caller packing) into the YA plane, which holds at least one field
        // (the masked inversion for members with land)
        e = run_prep(p, q, nullptr, 0, bc, s);
        if (!e) e = run_inversion(p, s);
        if (!e)
            e = timed(p, QG_K_OTHER, s, [&] {
                return launch_mode_to_layer(p->md, p->st_tiles, p->n_st, p->st_large, p->XC, p->YA, s, use_pdl(p));
            });
        psi = p->YA;
    }
    // stencil transposes: direct cotangent into S2, the adjoint solve's modal rhs into XB
    VjpArgs v = vjp_args(p);
    v.q = q;
    v.apply_bc = bc;
    v.psi = psi;
    v.gbar = dq_bar;
    v.params = params;
    v.direct = p->S2;
    v.rhs = p->XB;
    if (!e) e = cudaMemsetAsync(p->XB, 0, (size_t)p->xplane * sizeof(float), s);
    if (!e) e = timed(p, QG_K_STENCIL, s, [&] { return launch_vjp_stencil(v, s); });
    if (!e) e = timed(p, QG_K_PREP, s, [&] { return launch_vjp_operand(v, nullptr, s); });
    if (!e) e = run_inversion(p, s);  // the adjoint solve: the inversion is self-adjoint
    if (!e) e = timed(p, QG_K_OTHER, s, [&] { return launch_vjp_finish(v, p->XC, q_bar, nullptr, s); });
    return e;
}
}  // namespace

int qg_rhs_vjp(qg_plan* p, const float* q, const float* params, const float* dq_bar, float* q_bar,
               float* params_bar, int flags, void* stream) {
    if (!p || !q || !params || !dq_bar || !q_bar) return QG_ERR_NULL;
    if (flags & ~QG_RHS_APPLY_BC) return QG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const int bc = (flags & QG_RHS_APPLY_BC) ? 1 : 0;
    cudaError_t e = cudaMemsetAsync(p->vjp_acc, 0, (size_t)p->n_members * QG_NPARAMS * sizeof(double), s);
    if (!e) e = rhs_vjp_core(p, q, params, dq_bar, q_bar, bc, s);
    if (!e && params_bar) e = launch_vjp_params_only(vjp_args(p), params_bar, s);
    return cuda_err(e);
}

int64_t qg_step_vjp_workspace(const qg_plan* p, int scheme) {
    const Tableau* tb = swm_tableau(scheme);
    if (!p || !tb) return -1;
    return (int64_t)(4 * tb->n - 2) * p->state_size;
}

namespace {
// The launches of one step's adjoint (qg_step_vjp) on stream s.
cudaError_t step_vjp_body(qg_plan* p, const float* y0, const float* params, double dt, const Tableau* tb,
                          float* y_bar, float* params_bar, float* work, cudaStream_t s) {
    const int ns = tb->n;
    const int64_t n = p->state_size;
    // work: stage inputs Y_1 .. Y_{ns-1}, stage derivatives k_0 .. k_{ns-2}, their cotangents
    // kbar_0 .. kbar_{ns-1}, one stage-input cotangent Ybar, and the layer psi of the stage
    // inputs Y_0 .. Y_{ns-2} (from the recomputation, so that the reverse sweep inverts only
    // the last stage's input again)
    const float* Y[kMaxButcher];
    float* K[kMaxButcher];
    float* kbar[kMaxButcher];
    float* Psi[kMaxButcher];
    Y[0] = y0;
    for (int i = 1; i < ns; ++i) Y[i] = work + (int64_t)(i - 1) * n;
    for (int i = 0; i < ns - 1; ++i) K[i] = work + (int64_t)(ns - 1 + i) * n;
    for (int i = 0; i < ns; ++i) kbar[i] = work + (int64_t)(2 * ns - 2 + i) * n;
    float* Yb = work + (int64_t)(3 * ns - 2) * n;
    for (int i = 0; i < ns - 1; ++i) Psi[i] = work + (int64_t)(3 * ns - 1 + i) * n;
    // the step's stage inputs again: Y_s = y0 + dt sum_j a_sj k_j, k_j = F(B(Y_j))
    cudaError_t e = cudaSuccess;
    for (int st = 1; st < ns && !e; ++st) {
        e = rhs_core(p, Y[st - 1], K[st - 1], params, 1, s);
        // psi_hat of B(Y_{st-1}) is still in XC: keep its layer psi for the reverse sweep
        if (!e)
            e = timed(p, QG_K_OTHER, s, [&] {
                return launch_mode_to_layer(p->md, p->st_tiles, p->n_st, p->st_large, p->XC, Psi[st - 1], s,
                                            use_pdl(p));
            });
        float c[kMaxButcher];
        for (int j = 0; j < st; ++j) c[j] = (float)(dt * tb->a[st][j]);
        if (!e) e = launch_lincomb(const_cast<float*>(Y[st]), y0, K, c, st, n, s);
    }
    // reverse sweep: kbar_s = dt b_s g; per stage from the last, Ybar = F_vjp(Y_s; kbar_s),
    // then y_bar += Ybar and kbar_j += dt a_sj Ybar (j < s)
    if (!e) {
        float c[kMaxButcher];
        for (int j = 0; j < ns; ++j) c[j] = (float)(dt * tb->b[j]);
        e = launch_fanout(y_bar, kbar, c, ns, n, s);
    }
    if (!e) e = cudaMemsetAsync(p->vjp_acc, 0, (size_t)p->n_members * QG_NPARAMS * sizeof(double), s);
    for (int st = ns - 1; st >= 0 && !e; --st) {
        e = rhs_vjp_core(p, Y[st], params, kbar[st], Yb, 1, s, st < ns - 1 ? Psi[st] : nullptr);
        float c[kMaxButcher];
        for (int j = 0; j < st; ++j) c[j] = (float)(dt * tb->a[st][j]);
        if (!e) e = launch_scatter_bar(y_bar, Yb, kbar, c, st, n, s);
    }
    if (!e && params_bar) e = launch_vjp_params_only(vjp_args(p), params_bar, s);
    return e;
}
}  // namespace

int qg_step_vjp(qg_plan* p, const float* y0, const float* params, double dt, int scheme, float* y_bar,
                float* params_bar, float* work, void* stream) {
    if (!p || !y0 || !params || !y_bar || !work) return QG_ERR_NULL;
    const Tableau* tb = swm_tableau(scheme);
    if (!tb || !(dt == dt)) return QG_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    if (!p->opts.use_graphs || p->profiling)
        return cuda_err(step_vjp_body(p, y0, params, dt, tb, y_bar, params_bar, work, s));
    // a step's adjoint is ~10 launches per stage: captured once per set of arguments and
    // replayed as one graph while they repeat (callers that stage every step's state and
    // cotangent in the same buffers replay it every step)
    VjpGraph& g = p->vjp_graph;
    const void* ptr[5] = {y0, params, y_bar, params_bar, work};
    bool same = g.exec && g.dt == dt && g.scheme == scheme;
    for (int k = 0; k < 5 && same; ++k) same = g.ptr[k] == ptr[k];
    cudaError_t e = cudaSuccess;
    if (!same) {
        if (g.exec) {
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
        cudaGraph_t graph = nullptr;
        e = cudaStreamBeginCapture(p->cap, cudaStreamCaptureModeThreadLocal);
        if (!e) {
            const cudaError_t e1 = step_vjp_body(p, y0, params, dt, tb, y_bar, params_bar, work, p->cap);
            e = cudaStreamEndCapture(p->cap, &graph);
            if (!e) e = e1;
        }
        if (!e) e = cudaGraphInstantiate(&g.exec, graph, 0);
        if (graph) cudaGraphDestroy(graph);
        if (e) {
            g.exec = nullptr;
            return cuda_err(e);
        }
        for (int k = 0; k < 5; ++k) g.ptr[k] = ptr[k];
        g.dt = dt;
        g.scheme = scheme;
    }
    return cuda_err(cudaGraphLaunch(g.exec, s));
}

int qg_invert_vjp(qg_plan* p, const float* psi_bar, float* q_bar, void* stream) {
    if (!p || !psi_bar || !q_bar) return QG_ERR_NULL;
    cudaStream_t s = (cudaStream_t)stream;
    VjpArgs v = vjp_args(p);
    cudaError_t e = timed(p, QG_K_PREP, s, [&] { return launch_vjp_operand(v, psi_bar, s); });
    if (!e) e = run_inversion(p, s);  // self-adjoint, masked members included
    if (!e) e = timed(p, QG_K_OTHER, s, [&] { return launch_vjp_finish(v, p->XC, q_bar, nullptr, s); });
    return cuda_err(e);
}

int qg_diagnose(qg_plan* p, const float* q, float* ke, float* ens, void* stream) {
    if (!p || !q || !ke || !ens) return QG_ERR_NULL;
    cudaStream_t s = (cudaStream_t)stream;
    cudaError_t e = run_prep(p, q, nullptr, 0, 0, s);
    if (!e) e = run_inversion(p, s);
    if (!e) e = cudaMemsetAsync(p->diag_acc, 0, sizeof(double) * 2 * p->total_layers, s);
    if (!e)
        e = timed(p, QG_K_OTHER, s, [&] {
            return launch_diag_acc(p->md, p->st_tiles, p->n_st, p->st_large, q, p->XC, p->diag_acc, s);
        });
    if (!e) e = launch_diag_finish(p->diag_acc, p->total_layers, ke, ens, s);
    return cuda_err(e);
}

int qg_diagnose_fields(qg_plan* p, const float* q, float* psi, float* u, float* v, float* zeta, float* ke,
                       float* ens, void* stream) {
    if (!p || !q || !psi || !u || !v || !zeta || !ke || !ens) return QG_ERR_NULL;
    cudaStream_t s = (cudaStream_t)stream;
    // one inversion: psi_hat stays in XC for the KE reduction
    cudaError_t e = run_prep(p, q, nullptr, 0, 0, s);
    if (!e) e = run_inversion(p, s);
    if (!e)
        e = timed(p, QG_K_OTHER, s, [&] {
            return launch_mode_to_layer(p->md, p->st_tiles, p->n_st, p->st_large, p->XC, psi, s, false);
        });
    if (!e)
        e = timed(p, QG_K_OTHER, s, [&] {
            return launch_diag_fields(p->md, p->st_tiles, p->n_st, p->st_large, psi, u, v, zeta, s);
        });
    if (!e) e = cudaMemsetAsync(p->diag_acc, 0, sizeof(double) * 2 * p->total_layers, s);
    if (!e)
        e = timed(p, QG_K_OTHER, s, [&] {
            return launch_diag_acc(p->md, p->st_tiles, p->n_st, p->st_large, q, p->XC, p->diag_acc, s);
        });
    if (!e) e = launch_diag_finish(p->diag_acc, p->total_layers, ke, ens, s);
    return cuda_err(e);
}

int qg_state_stats(qg_plan* p, const float* q, double* stats, void* stream) {
    if (!p || !q || !stats) return QG_ERR_NULL;
    const int grid = std::max(1, std::min(p->n_sm * 4, (int)((p->state_size / 4 + 255) / 256)));
    return cuda_err(timed(p, QG_K_OTHER, (cudaStream_t)stream, [&] {
        return launch_state_stats(q, p->state_size, p->stats_acc, stats, grid, (cudaStream_t)stream);
    }));
}

int qg_status(qg_plan* p, int* flags, void* stream) {
    if (!p) return QG_ERR_NULL;
    cudaStream_t s = (cudaStream_t)stream;
    int h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, p->flags, sizeof(int), cudaMemcpyDeviceToHost, s);
    if (!e) e = cudaStreamSynchronize(s);
    if (!e) e = cudaMemsetAsync(p->flags, 0, sizeof(int), s);
    if (!e) e = cudaStreamSynchronize(s);
    if (e) return QG_ERR_CUDA;
    if (flags) *flags = h;
    if (h & 2) return QG_ERR_TIMEOUT;
    if (h & 4) return QG_ERR_CUDA;  // a kernel met a work item it was not built for and skipped it
    if (h & 1) return QG_ERR_NONFINITE;
    return QG_OK;
}

int qg_plan_set_parallel_sweep(qg_plan* p, int on) {
    if (!p) return QG_ERR_NULL;
    if (on != 0 && on != 1) return QG_ERR_ARG;
    if (p->fork_on != (on == 1)) {
        p->fork_on = on == 1;
        // the captured graphs hold the old launch structure
        cudaDeviceSynchronize();
        for (cudaGraphExec_t* x : {&p->graph.exec, &p->graph.exec_k, &p->vjp_graph.exec})
            if (*x) {
                cudaGraphExecDestroy(*x);
                *x = nullptr;
            }
    }
    return QG_OK;
}

int qg_plan_set_wait_limit(qg_plan* p, int64_t cycles) {
    if (!p) return QG_ERR_NULL;
    if (cycles < 0) return QG_ERR_ARG;
    p->pa.bar_wait = cycles == 0 ? kTimeoutCycles : (long long)cycles;
    return QG_OK;
}

int qg_plan_tuning(const qg_plan* p, int* variant, float* ms, int n) {
    if (!p) return QG_ERR_NULL;
    if (variant) *variant = p->sw_sel >= 0 ? 2 + p->sw_sel : p->st_large;
    for (int k = 0; ms && k < n && k < QG_STENCIL_VARIANTS; ++k) ms[k] = p->tune_ms[k];
    return QG_OK;
}

int qg_plan_gemm_tuning(const qg_plan* p, int* tile_n, float* ms, int n) {
    if (!p) return QG_ERR_NULL;
    if (tile_n) *tile_n = p->opts.dst_precision == QG_DST_FP32 ? kSimtBN : kGemmBN[p->bn_sel];
    for (int k = 0; ms && k < n && k < kNumBN; ++k) ms[k] = p->tune_gemm_ms[k];
    return QG_OK;
}

int qg_plan_engine(const qg_plan* p, int* cluster_ctas, float* ms, int n) {
    if (!p) return QG_ERR_NULL;
    if (cluster_ctas) *cluster_ctas = p->cl_use ? p->cl_C : 0;
    for (int k = 0; ms && k < n && k < 2; ++k) ms[k] = p->tune_engine_ms[k];
    return QG_OK;
}

int qg_set_profiling(qg_plan* p, int enable) {
    if (!p) return QG_ERR_NULL;
    cudaDeviceSynchronize();
    p->profiling = enable != 0;
    for (auto& u : p->ev_used) u = 0;
    return QG_OK;
}

int qg_kernel_stats(qg_plan* p, int k, double* total_ms, int64_t* launches) {
    if (!p || !total_ms || !launches) return QG_ERR_NULL;
    if (k < 0 || k >= QG_K_COUNT) return QG_ERR_ARG;
    double t = 0.0;
    for (size_t i = 0; i < p->ev_used[k]; ++i) {
        cudaEventSynchronize(p->ev[k][i].second);
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p->ev[k][i].first, p->ev[k][i].second) == cudaSuccess) t += ms;
    }
    *total_ms = t;
    *launches = (int64_t)p->ev_used[k];
    return QG_OK;
}

}  // extern "C"

namespace {

// Autotuner: time four SSP-RK3 steps of a zero state through qg_step with the multi-launch
// path (graph replay) and with the cluster engine, after one warm-up call each, and keep the
// faster.  The state is the YA plane (it holds at least one packed field), the parameters
// ones in the K planes.
int autotune_engine(qg_plan* p) {
    cudaStream_t s = p->cap;
    float* qd = p->YA;
    float* prm = p->K;
    std::vector<float> ones((size_t)p->n_members * QG_NPARAMS, 1.f);
    if (cudaMemsetAsync(qd, 0, sizeof(float) * p->state_size, s) ||
        cudaMemcpyAsync(prm, ones.data(), ones.size() * sizeof(float), cudaMemcpyHostToDevice, s) ||
        cudaStreamSynchronize(s))
        return QG_ERR_CUDA;
    cudaEvent_t e0, e1;
    if (cudaEventCreate(&e0)) return QG_ERR_CUDA;
    if (cudaEventCreate(&e1)) {
        cudaEventDestroy(e0);
        return QG_ERR_CUDA;
    }
    int r = QG_OK;
    for (int use = 0; use < 2 && r == QG_OK; ++use) {
        p->cl_use = use != 0;
        r = qg_step(p, qd, prm, 1200.0, 1, QG_SCHEME_SSPRK3, 0, s);
        if (r == QG_OK && cudaEventRecord(e0, s)) r = QG_ERR_CUDA;
        if (r == QG_OK) r = qg_step(p, qd, prm, 1200.0, 4, QG_SCHEME_SSPRK3, 0, s);
        float ms = -1.f;
        if (r == QG_OK && (cudaEventRecord(e1, s) || cudaEventSynchronize(e1) || cudaEventElapsedTime(&ms, e0, e1)))
            r = QG_ERR_CUDA;
        p->tune_engine_ms[use] = ms;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    p->cl_use = r == QG_OK && p->tune_engine_ms[1] >= 0.f && p->tune_engine_ms[1] < p->tune_engine_ms[0];
    int flags = 0;
    if (r == QG_OK) qg_status(p, &flags, s);  // clear what the timing runs left
    return r;
}

}  // namespace

namespace qg {
// Every scheme in Butcher form (the shallow-water stepper): Euler and Tsit5 as above, Heun
// (diffrax.Heun: c = [0, 1], b = [1/2, 1/2]) and the Shu-Osher SSP-RK3 (a21 = 1,
// a31 = a32 = 1/4, b = [1/6, 1/6, 2/3]).
const Tableau* swm_tableau(int scheme) {
    static const Tableau heun = {2, {{0, 0}, {1.0, 0}}, {0.5, 0.5}};
    static const Tableau ssprk3 = {3, {{0, 0, 0}, {1.0, 0, 0}, {0.25, 0.25, 0}}, {1.0 / 6.0, 1.0 / 6.0, 2.0 / 3.0}};
    if (scheme == QG_SCHEME_HEUN) return &heun;
    if (scheme == QG_SCHEME_SSPRK3) return &ssprk3;
    return butcher(scheme);
}
}  // namespace qg
