// qg_invert_static: the PV inversion of one member without a plan and without any device
// allocation.
//
// Who needs it: callers that may not allocate device memory at the time they invert, such
// as code running inside a framework's compiled program (an XLA custom call, a runtime
// that owns all device memory through its own pool), a real-time loop with an allocation
// ban, or a library that must not touch the process's allocator.  qg_plan_create
// allocates its constants and workspace with cudaMalloc; this entry point instead stages
// everything in one file-scope device array, g_qg_static_scratch, whose size is fixed at
// compile time (kScratchFloats floats, about 14.9 MB).  Every GPU that loads libqgcore.so
// holds that array until the process exits.
//
// Limits: Nx, Ny <= kStaticMaxN (interior nx, ny <= 512) and n_layers * Ny * round_up(Nx,
// 32) and n_layers * Nx * round_up(Ny, 32) each at most kStaticPlane floats (three layers of
// 514 x 514 fit).  Larger members are rejected with QG_ERR_TOO_LARGE before any launch.
//
// Sharing: all calls on a device use the same array and each call overwrites it, so calls
// whose kernels overlap on the GPU (different streams, or threads racing on one device)
// race on the scratch and give wrong results; serialise them.  Each call rebuilds every
// constant it reads (DST matrices, eigenvalues, member constants, tile lists) and writes
// every plane element before reading it, so nothing left by an earlier call is read.
//
// First call on a device: the host looks up the array's device address with
// cudaGetSymbolAddress (once per device and context, with that device current) and caches
// it together with the context's unique id.  Make that first call outside any stream
// capture.  A later call in a new context of the device (after cudaDeviceReset, whose
// module reload can move the array) sees a different id and looks the address up again.
#include <cuda.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "qg_internal.cuh"

namespace qg {
namespace {

constexpr int kStaticMaxN = 514;
constexpr int kStaticMaxP = 544;                     // round_up(514, 32)
constexpr int64_t kStaticPlane = 1 << 20;            // floats per workspace plane
constexpr int kStaticMaxTiles = 4096;                // per tile list
constexpr int64_t kMemberFloats = 512;               // >= sizeof(MemberDev) / 4
constexpr int64_t kOffPlanes = 0;                                      // 3 planes
constexpr int64_t kOffSx = kOffPlanes + 3 * kStaticPlane;              // Nx x Px
constexpr int64_t kOffSy = kOffSx + (int64_t)kStaticMaxN * kStaticMaxP; // Ny x Py
constexpr int64_t kOffEig = kOffSy + (int64_t)kStaticMaxN * kStaticMaxP; // ex, ey
constexpr int64_t kOffMember = kOffEig + 2 * kStaticMaxP;
constexpr int64_t kOffTiles = kOffMember + kMemberFloats;              // 3 lists x 3 ints
constexpr int64_t kScratchFloats = kOffTiles + 3 * 3 * (int64_t)kStaticMaxTiles;

static_assert(sizeof(MemberDev) <= kMemberFloats * 4, "member constants do not fit");
static_assert(sizeof(StencilTile) == 12 && sizeof(GemmTile) == 12, "tile layout");

// The scratch.  Host code never dereferences this symbol: on the host it names a stand-in,
// not the device array, so its device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) float g_qg_static_scratch[kScratchFloats];

std::mutex g_mu;
float* g_base[64] = {nullptr};
unsigned long long g_ctx_id[64] = {0};

using CtxGetCurrent = CUresult (*)(CUcontext*);
using CtxGetId = CUresult (*)(CUcontext, unsigned long long*);
CtxGetCurrent g_ctx_current = nullptr;
CtxGetId g_ctx_get_id = nullptr;
bool g_ctx_fn_tried = false;

// Unique id of the current context (0 when the driver cannot say; the address is then
// looked up on every call).  Called with g_mu held.
unsigned long long current_context_id() {
    if (!g_ctx_fn_tried) {
        g_ctx_fn_tried = true;
        void* f1 = nullptr;
        void* f2 = nullptr;
        cudaDriverEntryPointQueryResult q1, q2;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f1, 12000, cudaEnableDefault, &q1) == cudaSuccess &&
            q1 == cudaDriverEntryPointSuccess &&
            cudaGetDriverEntryPointByVersion("cuCtxGetId", &f2, 12000, cudaEnableDefault, &q2) == cudaSuccess &&
            q2 == cudaDriverEntryPointSuccess && f1 && f2) {
            g_ctx_current = reinterpret_cast<CtxGetCurrent>(f1);
            g_ctx_get_id = reinterpret_cast<CtxGetId>(f2);
        }
    }
    if (!g_ctx_current || !g_ctx_get_id) return 0;
    CUcontext ctx = nullptr;
    unsigned long long id = 0;
    if (g_ctx_current(&ctx) != CUDA_SUCCESS || !ctx || g_ctx_get_id(ctx, &id) != CUDA_SUCCESS) return 0;
    return id;
}

// Device address of the scratch on the current device, looked up once per device and
// context.
cudaError_t scratch_base(float** out) {
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    if (dev < 0 || dev >= 64) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lk(g_mu);
    const unsigned long long id = current_context_id();
    if (!g_base[dev] || id == 0 || id != g_ctx_id[dev]) {
        void* p = nullptr;
        e = cudaGetSymbolAddress(&p, g_qg_static_scratch);
        if (e != cudaSuccess) return e;
        g_base[dev] = static_cast<float*>(p);
        g_ctx_id[dev] = current_context_id();  // the lookup made the device's context current
    }
    *out = g_base[dev];
    return cudaSuccess;
}

// Rebuild every constant of the member inside the scratch: the member record (with its
// device pointers into the scratch), the orthonormal DST-I matrices, their eigenvalues and
// the stencil / GEMM tile lists.
__global__ void k_static_setup(MemberDev M, double dx, double dy, float* base, int n_st, int st_tx, int n_gx,
                               int gx_nt, int n_gy, int gy_nt) {
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    if (tid == 0) *reinterpret_cast<MemberDev*>(base + kOffMember) = M;
    auto fill_dst = [&](float* S, int n, int ld) {
        const double s = sqrt(2.0 / (n + 1));
        const long long per = 2LL * (n + 1);
        for (int64_t k = tid; k < (int64_t)n * n; k += nth) {
            const int i = (int)(k / n), j = (int)(k % n);
            const long long a = ((long long)(i + 1) * (j + 1)) % per;
            S[(int64_t)i * ld + j] = (float)(s * sinpi((double)a / (n + 1)));
        }
    };
    fill_dst(base + kOffSx, M.Nx, M.Px);
    fill_dst(base + kOffSy, M.Ny, M.Py);
    for (int64_t k = tid; k < M.Nx + M.Ny; k += nth) {
        const bool xdir = k < M.Nx;
        const int n = xdir ? M.Nx : M.Ny;
        const int kk = (int)(xdir ? k : k - M.Nx) + 1;
        const double d = xdir ? dx : dy;
        const double sn = sinpi((double)kk / (2.0 * (n + 1)));
        (base + kOffEig)[xdir ? k : kStaticMaxP + (k - M.Nx)] = (float)(-4.0 * sn * sn / (d * d));
    }
    int* tiles = reinterpret_cast<int*>(base + kOffTiles);
    for (int64_t t = tid; t < n_st; t += nth) {
        StencilTile* st = reinterpret_cast<StencilTile*>(tiles);
        st[t] = {0, (int)(t / st_tx), (int)(t % st_tx)};
    }
    for (int64_t t = tid; t < n_gx; t += nth) {
        GemmTile* g = reinterpret_cast<GemmTile*>(tiles + 3 * kStaticMaxTiles);
        g[t] = {0, (int)(t / gx_nt), (int)(t % gx_nt)};
    }
    for (int64_t t = tid; t < n_gy; t += nth) {
        GemmTile* g = reinterpret_cast<GemmTile*>(tiles + 6 * kStaticMaxTiles);
        g[t] = {0, (int)(t / gy_nt), (int)(t % gy_nt)};
    }
}

}  // namespace
}  // namespace qg

using namespace qg;

extern "C" int qg_invert_static(const qg_member_desc* member, const float* q, float* psi, void* stream) {
    if (!member || !q || !psi) return QG_ERR_NULL;
    const qg_member_desc& d = *member;
    if (d.mask) return QG_ERR_UNSUPPORTED;  // land needs the plan's capacitance matrices
    const int v = validate_member(d);
    if (v != QG_OK) return v;
    const int Ny = d.ny + 2, Nx = d.nx + 2, nl = d.n_layers;
    const int Px = round_up(Nx, 32), Py = round_up(Ny, 32);
    if (Nx > kStaticMaxN || Ny > kStaticMaxN) return QG_ERR_TOO_LARGE;
    if ((int64_t)nl * Ny * Px > kStaticPlane || (int64_t)nl * Nx * Py > kStaticPlane) return QG_ERR_TOO_LARGE;
    const int st_ty = (Ny + kTileSY - 1) / kTileSY, st_tx = (Nx + kTileSX - 1) / kTileSX;
    const int gx_mt = (nl * Ny + kSimtBM - 1) / kSimtBM, gx_nt = (Nx + kSimtBN - 1) / kSimtBN;
    const int gy_mt = (nl * Nx + kSimtBM - 1) / kSimtBM, gy_nt = (Ny + kSimtBN - 1) / kSimtBN;
    const int n_st = st_ty * st_tx, n_gx = gx_mt * gx_nt, n_gy = gy_mt * gy_nt;
    if (n_st > kStaticMaxTiles || n_gx > kStaticMaxTiles || n_gy > kStaticMaxTiles) return QG_ERR_TOO_LARGE;

    float* base = nullptr;
    if (scratch_base(&base) != cudaSuccess) return QG_ERR_CUDA;
    cudaStream_t s = (cudaStream_t)stream;

    MemberDev M;
    double Cl2m[64], Cm2l[64], lam[8];
    member_constants(d, M, Cl2m, Cm2l, lam);
    // one member: the caller's fields start at 0; the x-row and y-row planes are three
    // scratch planes reused in turn (modal q -> T1t -> U -> Vt -> psi_hat)
    M.off_state = M.off_x = M.off_y = M.off_layer = 0;
    M.ex = base + kOffEig;
    M.ey = base + kOffEig + kStaticMaxP;
    M.Sx = base + kOffSx;
    M.Sy = base + kOffSy;
    float* P0 = base + kOffPlanes;
    float* P1 = P0 + kStaticPlane;
    float* P2 = P1 + kStaticPlane;
    const MemberDev* md = reinterpret_cast<const MemberDev*>(base + kOffMember);
    const int* tiles = reinterpret_cast<const int*>(base + kOffTiles);
    const StencilTile* st = reinterpret_cast<const StencilTile*>(tiles);
    const GemmTile* gx = reinterpret_cast<const GemmTile*>(tiles + 3 * kStaticMaxTiles);
    const GemmTile* gy = reinterpret_cast<const GemmTile*>(tiles + 6 * kStaticMaxTiles);

    k_static_setup<<<64, 256, 0, s>>>(M, d.Lx / d.nx, d.Ly / d.ny, base, n_st, st_tx, n_gx, gx_nt, n_gy, gy_nt);
    cudaError_t e = cudaGetLastError();
    if (!e) {
        PrepArgs pa{};
        pa.members = md;
        pa.tiles = st;
        pa.q = q;
        pa.xa = P0;
        pa.xa_fmt = FMT_F32;
        pa.xplane = kStaticPlane;
        pa.tile_x = kTileSX;
        pa.tile_y = kTileSY;
        e = launch_prep(pa, n_st, s, false);
    }
    auto gemm = [&](int pass, const float* A, float* C, const GemmTile* tl, int nt) {
        GemmArgs g{};
        g.members = md;
        g.xplane = g.yplane = kStaticPlane;
        g.tiles = tl;
        g.pass = pass;
        g.A = A;
        g.C = C;
        g.a_fmt = g.c_fmt = FMT_F32;
        return launch_gemm_simt(g, nt, s, false);
    };
    if (!e) e = gemm(G1_FWD_X, P0, P1, gx, n_gx);
    if (!e) e = gemm(G2_FWD_Y, P1, P2, gy, n_gy);
    if (!e) e = gemm(G3_INV_X, P2, P0, gx, n_gx);
    if (!e) e = gemm(G4_INV_Y, P0, P1, gy, n_gy);
    if (!e) e = launch_mode_to_layer(md, st, n_st, 0, P1, psi, s, false);
    return e == cudaSuccess ? QG_OK : QG_ERR_CUDA;
}
