// Internal declarations shared by the libqgcore translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <utility>
#include <vector>

#include "../../include/qgcore.h"

namespace qg {

constexpr int kMaxLayers = QG_MAX_LAYERS;

// Per-member constants, resident in device memory (an array indexed by member id) so that
// one launch can serve every member of an ensemble.
struct MemberDev {
    int nl, Ny, Nx;
    int Px, Py;      // padded pitches (floats): x-row planes (nl, Ny, Px), y-row planes (nl, Nx, Py)
    int barotropic;  // BarotropicQG semantics
    float dx, dy;
    float inv_dx2, inv_dy2;
    float inv_12dxdy;  // 1 / (12 dx dy): Arakawa normalisation
    float beta_12dx;   // beta / (12 dx): the beta-term of J(psi, beta y) for a linear beta y
    float invH0;       // 1 / H[0] (1 for barotropic)
    float f0;          // Coriolis parameter
    float H[kMaxLayers];  // layer thicknesses (the geostrophic projection)
    float Cl2m[kMaxLayers * kMaxLayers];
    float Cm2l[kMaxLayers * kMaxLayers];
    float lam[kMaxLayers];  // f0^2 * eig
    int64_t off_state;      // offset (floats) of this member in a caller's packed field
    int64_t off_x;          // offset (floats) in the internal x-row planes
    int64_t off_y;          // offset (floats) in the internal y-row planes
    int64_t off_layer;      // offset of this member's first layer in per-layer outputs
    const float* by;        // beta * (y_j - Ly/2), Ny
    const float* F;         // wind pattern, Ny
    const float* ex;        // DST-I eigenvalues along x (Nx)
    const float* ey;        // along y (Ny)
    const float* Sx;        // orthonormal DST-I matrix Nx x Nx, pitch Px
    const float* Sy;        // Ny x Ny, pitch Py
    const uint16_t* Sx_bf;  // bf16 hi/lo planes of Sx (pitch Px, hi then lo), or null
    const uint16_t* Sy_bf;
    // masked basin (null / 0 without land)
    const uint8_t* mask;    // (Ny, Nx), 1 = ocean; interior cells with 0 are land
    int nb;                 // land boundary points B (capacitance correction)
    const int* bidx;        // their linear indices j * Nx + i
    const double* cinv;     // nl x nb x nb inverse capacitance matrices (row-major)
};

// Interior land cell of a member (false without a mask).
__host__ __device__ __forceinline__ bool is_land(const uint8_t* mask, int Ny, int Nx, int j, int i) {
    return mask && j > 0 && i > 0 && j < Ny - 1 && i < Nx - 1 && mask[(int64_t)j * Nx + i] == 0;
}
__host__ __device__ __forceinline__ bool is_land(const MemberDev& M, int j, int i) {
    return is_land(M.mask, M.Ny, M.Nx, j, i);
}

// Stencil work item: one 2-D tile of one member (all layers).
struct StencilTile {
    int member, ty, tx;
};

// GEMM work item: one output tile of one member for one pass.
struct GemmTile {
    int member, mt, nt;
};

// The four DST-I GEMM passes of the inversion, psi_hat = S_y (S_y q S_x ./ L) S_x.
// Each is C = A * S with A row-major (rows = (layer, r), K contiguous) and S symmetric, stored
// transposed (C^T = S A^T), so the contracted axis alternates x, y, x, y and the last pass
// leaves psi_hat in the x-row layout of q.  Every store is column-major in C: the lanes of a
// warp hold consecutive rows of the accumulator and write consecutive addresses.
enum GemmPass : int {
    G1_FWD_X = 0,  // A = q_modal rows (l, y), K = x  -> T1[l][kx][y]              (y-row plane)
    G2_FWD_Y = 1,  // A = T1 rows (l, kx), K = y      -> U[l][ky][kx] / (ex+ey-lam) (x-row plane)
    G3_INV_X = 2,  // A = U rows (l, ky), K = kx      -> V[l][x][ky]               (y-row plane)
    G4_INV_Y = 3,  // A = V rows (l, x), K = ky       -> psi_hat[l][y][x]          (x-row plane)
};
// A of the pass is an x-row plane (rows (l, y), K = x); its output is then a y-row plane.
__host__ __device__ constexpr bool pass_xin(int pass) { return pass == G1_FWD_X || pass == G3_INV_X; }

// Operand / output formats of the internal planes.
enum PlaneFmt : int {
    FMT_F32 = 0,     // float32 plane
    FMT_BF16X2 = 1,  // bf16 hi plane followed by bf16 lo plane (same byte size as f32)
};

// Programmatic-dependent-launch-capable launch: with `pdl` the kernel may start while its
// predecessor in the stream finishes; every kernel calls griddepcontrol.wait before it
// touches memory a predecessor writes.
template <typename... KArgs, typename... Args>
cudaError_t launch_k(void (*kernel)(KArgs...), int grid, int block, size_t smem, cudaStream_t s, bool pdl,
                     Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

// Butcher tableau of an explicit Runge-Kutta scheme: a[s][j] (j < s) and b[s], n stages.
constexpr int kMaxButcher = 6;
struct Tableau {
    int n;
    double a[kMaxButcher][kMaxButcher];
    double b[kMaxButcher];
};

struct PrepArgs {
    const MemberDev* members;
    const StencilTile* tiles;
    const float* q;        // caller packing
    float* copy;           // internal x-row plane to receive q (may be null)
    int zero_ring_copy;    // zero the ring in the copy
    int bc_operand;        // operand built from q with a zero ring
    void* xa;              // Cl2m q in the GEMM operand format (may be null)
    int xa_fmt;
    float* xq;             // FP32 Cl2m q for the refinement residual (may be null)
    int64_t xplane;
    int tile_x, tile_y;    // cells per tile of the tile list
};

// Butcher-form stage combine: out = y0 + dt * sum_s coef[s] * k[s] and its modal operand.
constexpr int kMaxStages = 8;
struct RkCombineArgs {
    const MemberDev* members;
    const StencilTile* tiles;
    int tile_x, tile_y;
    const float* y0;       // x-row state plane
    const float* k;        // stage derivatives, caller packing, plane s at s * kplane
    int64_t kplane;
    int n_k;
    float coef[kMaxStages];
    float dt;
    float* out;            // x-row stage plane (the next stage input or the new state)
    void* xa;              // modal operand of `out` (zero ring and land)
    int xa_fmt;
    float* xq;             // its FP32 copy (refinement), or null
    int64_t xplane;
};
cudaError_t launch_rk_combine(const RkCombineArgs& a, int ntiles, cudaStream_t s, bool pdl);

// TMA descriptors of one member for the stencil: the three stage planes and psi_hat,
// 3-D boxes (x, y, layer) over the padded x-row planes.
constexpr int kStencilMapsBytes = 4 * 128;
cudaError_t stencil_encode_maps(const MemberDev& M, const float* const planes[4], int large, void* out);

struct StencilArgs {
    const MemberDev* members;
    const StencilTile* tiles;
    const void* maps;      // StencilMaps per member
    int q_sel;             // which stage plane holds the input q (0..2)
    const float* params;   // n_members * QG_NPARAMS
    int apply_bc;          // zero the ring of q on read
    int64_t xplane;
    // rhs mode
    float* dq;             // caller packing; null in step mode
    // step mode: y_next = a * y0 + b * (y_s + dt * dq), internal planes
    const float* y0;
    float* y_next;
    int final_stage;
    float a, b, dt;
    void* xa;              // next-stage GEMM operand (modal q, x-row planes); may be null
    int xa_fmt;
    float* xq;             // FP32 copy of the modal q for the refinement residual; may be null
    int* flags;            // device status word
    // the column-sweep stencil reads the planes directly
    const float* qin;      // stage plane holding the input q (x-row)
    const float* psi_hat;  // psi_hat plane (x-row)
};

// Work item of the column-sweep stencil: strip sx (28 output columns) of row block sy.
struct SweepItem {
    int member, sx, sy;
};
int sweep_columns();
int sweep_warps_per_block();
int sweep_blocks_per_sm(int nl);
// one launch per layer count k + 1 with n_items[k] > 0 (items grouped by layer count)
cudaError_t launch_sweep(const StencilArgs& a, const SweepItem* const* items, const int* n_items, int R,
                         const int* grid, cudaStream_t s, bool pdl);
// The layer-per-warp sweep (two columns per lane, one warp per layer of a strip): items are
// strips of kLSweepOut output columns, lsweep_strips_per_block(nl) strips per CTA.  Each strip
// class has its own kernel: 0 = every column and row the strip reads is strictly inside the
// member (no ring, member-edge or store predicates), 1 = the strip touches the ring or the
// member's edge in x and in y, 2 = masked member (land rules), 3 = it touches them in x only
// (its rows are strictly inside), 4 = in y only (its columns are strictly inside).
constexpr int kLSweepOut = 60;
constexpr int kLSweepClasses = 5;
// Row bands of a member's strips: band sy covers rows [sy R, lsweep_band_end).  A remainder of
// fewer than kLSweepAbsorb rows below the last full band is absorbed into that band (while it
// stays within the 64 rows whose wind a strip holds in registers), so that no strip pays a
// whole strip's start-up for a few rows (every square member of N = n + 2 with n a multiple
// of 32 would otherwise end in a 2-row band).
constexpr int kLSweepAbsorb = 8;
__host__ __device__ inline int lsweep_bands(int Ny, int R) {
    int n = (Ny + R - 1) / R;
    const int rem = Ny - (n - 1) * R;
    if (n > 1 && rem < kLSweepAbsorb && R + rem <= 64) --n;
    return n;
}
__host__ __device__ inline int lsweep_band_end(int Ny, int sy, int R) {
    return sy + 1 >= lsweep_bands(Ny, R) ? Ny : (sy + 1) * R;
}
__host__ __device__ inline int lsweep_item_class(int Ny, int Nx, bool masked, int sx, int sy, int R) {
    if (masked) return 2;
    const int x0 = sx * kLSweepOut, jb = sy * R, rhi = lsweep_band_end(Ny, sy, R) + 1;
    // columns x0 - 2 .. x0 + 61 and rows jb - 2 .. rhi are read
    const bool xin = x0 - 2 >= 1 && x0 + 61 <= Nx - 2, yin = jb - 2 >= 1 && rhi <= Ny - 2;
    return xin ? (yin ? 0 : 4) : (yin ? 3 : 1);
}
int lsweep_columns();
int lsweep_strips_per_block(int nl);
int lsweep_blocks_per_sm(int nl, int cls);
// items / n_items / grid: kMaxLayers * kLSweepClasses groups, group (nl - 1) * kLSweepClasses + class
cudaError_t launch_lsweep(const StencilArgs& a, const SweepItem* const* items, const int* n_items, int R,
                          const int* grid, cudaStream_t s, bool pdl);
// one (layer count, strip class) group g of launch_lsweep
cudaError_t launch_lsweep_group(const StencilArgs& a, const SweepItem* items, int n_items, int R, int grid, int g,
                                cudaStream_t s, bool pdl);

// launchers (return cudaError_t of the launch)
cudaError_t launch_prep(const PrepArgs& a, int ntiles, cudaStream_t s, bool pdl);
cudaError_t launch_unpack(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                          const float* src, float* q, cudaStream_t s, bool pdl);
cudaError_t launch_mode_to_layer(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                                 const float* psi_hat, float* psi, cudaStream_t s, bool pdl);
cudaError_t launch_diag_acc(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                            const float* q, const float* psi_hat, double* acc, cudaStream_t s);
// min / mean / max of the finite entries and the non-finite count of n floats into out[0..3]
// (device doubles); acc: 32 bytes of device scratch
cudaError_t launch_state_stats(const float* q, int64_t n, void* acc, double* out, int grid, cudaStream_t s);
cudaError_t launch_diag_fields(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                               const float* psi, float* u, float* v, float* zeta, cudaStream_t s);
cudaError_t launch_diag_finish(const double* acc, int64_t n_layers, float* ke, float* ens,
                               cudaStream_t s);
// geostrophic projection of a shallow-water state (h, u, v): the PV q in front of the
// inversion, then (h_g, u_g, v_g) from psi
cudaError_t launch_project_q(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                             const float* h, const float* u, const float* v, float* q, cudaStream_t s);
cudaError_t launch_project_g(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                             const float* psi, float* hg, float* ug, float* vg, cudaStream_t s);
cudaError_t launch_project_g_vjp(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                                 const float* hgb, const float* ugb, const float* vgb, float* psib, cudaStream_t s);
cudaError_t launch_project_q_vjp(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                                 const float* qb, float* hb, float* ub, float* vb, cudaStream_t s);
cudaError_t launch_residual(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                            const float* qm, const float* psi_hat, void* out, int out_fmt,
                            int64_t xplane, cudaStream_t s, bool pdl);

// Adjoint (qg_adjoint.cu): the RHS / inversion VJP around one adjoint DST solve.
struct VjpArgs {
    const MemberDev* members;
    const StencilTile* tiles;
    int ntiles, tile_x, tile_y, max_nl, n_members;
    const float* q;       // caller packing
    int apply_bc;         // the forward zeroed the ring of q on read
    const float* psi;     // layer psi of the forward, caller packing
    const float* gbar;    // cotangent of dq, caller packing
    const float* params;  // n_members * QG_NPARAMS
    float* direct;        // x-row plane: cotangent of qb from the stencil terms (null: none)
    float* rhs;           // FP32 x-row modal plane: Cm2l^T Z psi_bar (zeroed before the stencil)
    double* pacc;         // parameter cotangents (zeroed before the stencil)
    void* xa;             // GEMM operand of the adjoint solve
    int xa_fmt;
    float* xq;            // its FP32 copy for the refinement residual (may be null)
    int64_t xplane;
};
cudaError_t launch_vjp_stencil(const VjpArgs& v, cudaStream_t s);
cudaError_t launch_vjp_operand(const VjpArgs& v, const float* psi_bar, cudaStream_t s);
cudaError_t launch_vjp_finish(const VjpArgs& v, const float* xbar, float* qbar, float* pbar, cudaStream_t s);
cudaError_t launch_vjp_params_only(const VjpArgs& v, float* pbar, cudaStream_t s);
// out = base + sum_j c_j x_j; ybar += Yb, kbar_j += c_j Yb; out_j = c_j g (n floats each)
cudaError_t launch_lincomb(float* out, const float* base, const float* const* x, const float* c, int n_terms,
                           int64_t n, cudaStream_t s);
cudaError_t launch_scatter_bar(float* ybar, const float* Yb, float* const* kbar, const float* c, int n_terms,
                               int64_t n, cudaStream_t s);
cudaError_t launch_fanout(const float* g, float* const* out, const float* c, int n_terms, int64_t n, cudaStream_t s);
const Tableau* swm_tableau(int scheme);

// host: cuTensorMapEncodeTiled through the driver entry point (no libcuda link needed)
cudaError_t tmap_encode(void* map, int bf16, int rank, const void* base, const uint64_t* dims,
                        const uint64_t* strides_bytes, const uint32_t* box, int swizzle128);

struct GemmArgs {
    const MemberDev* members;
    int64_t xplane, yplane;  // elements of one x-row / y-row plane (bf16 lo-plane offset)
    const GemmTile* tiles;
    int pass;
    const void* A;   // plane base (internal packing)
    void* C;         // plane base
    int a_fmt, c_fmt;
    int accumulate;       // C += result (refinement of psi_hat)
    const void* tc_maps;  // tensor-core path: TMA descriptors, 4 per member (one per pass)
    int* flags;           // device status word (bit 1: a bounded wait timed out)
};
constexpr int kTcMapsBytes = 512;

// Arguments of the persistent step kernel (qg_persistent.cu).
struct PersistArgs {
    const MemberDev* members;
    const GemmTile* gx;
    const GemmTile* gy;
    const StencilTile* st;
    int n_gx, n_gy, n_st, max_nl;
    int tile_n;               // DST GEMM output tile width (<= TC_BN, a multiple of 16)
    const void* tc_maps;
    const void* st_maps;
    void *XA, *YA, *YB, *XB;  // operand-format planes
    float* XC;                // psi_hat
    float* S[3];              // stage planes (S[0] = state)
    const float* params;
    int64_t xplane, yplane;
    size_t slot_bytes;        // one stencil box buffer (q and psi boxes)
    size_t lap_offset;        // shared-memory offset of the lap(q) buffer
    int st_nbuf;              // stencil box buffers (2: next tile loads during compute)
    int st_large;             // stencil tile shape: 0 = 32 x 8, 1 = 64 x 16
    int g4_accumulate;        // the last GEMM pass adds into psi_hat (refinement)
    int op_fmt;
    int n_stages, n_steps;
    float sa[4], sb[4], dt;   // Shu-Osher stage coefficients
    int* flags;
    unsigned* bar_count;      // grid barrier: arrivals, generation (zeroed before every launch)
    unsigned* bar_gen;
    long long bar_wait;       // clock64 cycles a CTA waits at the grid barrier before giving up
};
size_t persistent_smem_bytes(int precision, int max_nl, int large, PersistArgs* a);
cudaError_t persistent_init();
cudaError_t launch_persistent(const PersistArgs& a, int grid, int precision, cudaStream_t s);
// multi-tile stand-alone launches (the graph-captured multi-launch path)
cudaError_t launch_gemm_mt(const PersistArgs& a, int pass, int grid, int precision, cudaStream_t s, bool pdl);
cudaError_t launch_stencil_mt(const StencilArgs& sa, int n_st, int grid, int max_nl, int large, cudaStream_t s,
                              bool pdl);
int stencil_mt_blocks_per_sm(int max_nl, int large);  // 4 CUtensorMap per (member, pass)
cudaError_t gemm_tc_encode(const MemberDev& M, int pass, const void* a_plane, int64_t a_plane_elems, int prec,
                           void* out);
cudaError_t launch_gemm_simt(const GemmArgs& g, int ntiles, cudaStream_t s, bool pdl);

// masked basins: host construction (qg_capacitance.cu) and the device correction (qg_mask.cu)
struct CapItem {
    int member, mode, r0;  // rows r0 .. r0 + kCapRows - 1 of C^-1 of one mode
};
constexpr int kCapRows = 32;
std::vector<int> land_boundary(const qg_member_desc& d);
bool capacitance_inverse(const qg_member_desc& d, const double* lam, int nl, const std::vector<int>& B,
                         std::vector<double>& cinv);
// sigma = -C^-1 psi_hat[B] per (member, mode), written at B into the operand (and its FP32
// copy) for the second solve
cudaError_t launch_capacitance(const MemberDev* members, const CapItem* items, int n_items, const float* psi_hat,
                               void* xa, int xa_fmt, float* xq, int64_t xplane, size_t smem, cudaStream_t s);
cudaError_t capacitance_init(size_t max_smem);
constexpr int kMaxBoundary = 28000;  // boundary points per member (FP64 gather in shared memory)

// Cluster-resident stepping of small members (qg_cluster.cu): shared-memory layout of one
// CTA of a cluster of C CTAs for a member of nl layers on an Ny x Nx grid (float offsets).
struct ClGeom {
    int C, By, Bx;         // row / column block of a CTA
    int BPy, BPx;          // blocks padded to a multiple of 4
    int BPe, BPq;          // row block + 1-row halos (psi, lap q), + 2-row halos (stage input)
    int Hx, Hy, NPx, NPy;  // folded DST-I matrices: ceil(N / 2) rows, pitch round_up(N, 4)
    int share_s;           // Nx == Ny: one matrix for both axes
    int o_sx, o_sy, o_ra, o_rb, o_psi, o_fold, o_q0, o_q1, o_y0, o_stg, o_const, total;
};
__host__ __device__ inline int round4(int v) { return (v + 3) & ~3; }
__host__ __device__ inline ClGeom cl_geom(int nl, int Ny, int Nx, int C) {
    ClGeom g;
    g.C = C;
    g.By = (Ny + C - 1) / C;
    g.Bx = (Nx + C - 1) / C;
    g.BPy = round4(g.By);
    g.BPx = round4(g.Bx);
    g.BPe = round4(g.By + 2);
    g.BPq = round4(g.By + 4);
    g.Hx = (Nx + 1) / 2;
    g.Hy = (Ny + 1) / 2;
    g.NPx = round4(Nx);
    g.NPy = round4(Ny);
    g.share_s = Nx == Ny;
    int o = 0;
    g.o_sx = o;
    o += g.Hx * g.NPx;
    g.o_sy = g.share_s ? g.o_sx : o;
    if (!g.share_s) o += g.Hy * g.NPy;
    g.o_ra = o;  // x-owned planes [nl][Ny][BPx]
    o += nl * Ny * g.BPx;
    g.o_rb = o;  // y-owned planes [nl][Nx][BPy] (also the operand of the first pass)
    o += nl * Nx * g.BPy;
    g.o_psi = o;  // psi_hat / psi with 1-row halos [nl][Nx][BPe]
    o += nl * Nx * g.BPe;
    const int Hm = g.Hx > g.Hy ? g.Hx : g.Hy, BPm = g.BPx > g.BPy ? g.BPx : g.BPy;
    const int fold = nl * Hm * 2 * BPm, lap = nl * Nx * g.BPe;
    g.o_fold = o;  // folded pass input; lap q during the stencil
    o += fold > lap ? fold : lap;
    g.o_q0 = o;  // stage inputs with 2-row halos [nl][Nx][BPq], two
    o += nl * Nx * g.BPq;
    g.o_q1 = o;
    o += nl * Nx * g.BPq;
    g.o_y0 = o;  // state [nl][Nx][BPy]
    o += nl * Nx * g.BPy;
    const int Bm = g.By > g.Bx ? g.By : g.Bx;
    const int BPo = BPm > g.BPe ? BPm : g.BPe;
    g.o_stg = o;  // outgoing chunks [C][nl][rows][BPo]
    o += C * nl * Bm * BPo;
    g.o_const = o;  // Cm2l, Cl2m (nl x nl), lambda (nl), F (Ny), ex (Nx), ey (Ny)
    o += round4(2 * nl * nl + nl + 2 * Ny + Nx);
    g.total = o;
    return g;
}
int cluster_size_for(int nl, int Ny, int Nx, size_t* smem_bytes);
cudaError_t launch_cluster(const MemberDev* members, int n_members, int nl, int C, size_t smem, float* q,
                           const float* params, int apply_bc, int n_steps, int n_stages, const float* sa,
                           const float* sb, float dt, int* flags, cudaStream_t s);

// host helpers shared by the plan and the plan-free entry points
int validate_member(const qg_member_desc& d);
void member_constants(const qg_member_desc& d, MemberDev& M, double* Cl2m, double* Cm2l, double* lam);
int round_up(int v, int m);

// stencil tile shapes (cells): small grids use 32 x 8, large ones 64 x 16
constexpr int kTileSX = 32, kTileSY = 8, kTileLX = 64, kTileLY = 16;
constexpr int kSimtBM = 64;
constexpr int kSimtBN = 64;

}  // namespace qg
