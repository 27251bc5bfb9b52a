// Memory-bound kernels of the QG time step: the fused RHS stencil (with the RK stage update
// and the next stage's layer->mode prologue fused in), the pack / unpack of the state into
// the padded internal planes, the mode->layer epilogue, the Helmholtz residual and the
// diagnostics.
//
// Every kernel walks a list of 2-D tiles (StencilTile) that may belong to different members
// of an ensemble; a block owns one tile and all layers of it.  Kernels start with the
// programmatic-dependent-launch handshake: constants are read before griddepcontrol.wait,
// anything a predecessor kernel writes only after it.
#include <cuda_bf16.h>

#include <cstring>

#include "qg_stencil_tile.cuh"

namespace qg {

using namespace st;

// ---------------------------------------------------------------------------------------
// Pack: copy q (caller packing) into an internal plane (optionally zeroing its ring) and
// write the layer->mode operand Cl2m q (BC applied when bc_operand) for the DST GEMMs.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_prep(PrepArgs a) {
    __shared__ MemberDev M;
    const StencilTile t = a.tiles[blockIdx.x];
    const int TX = a.tile_x, TY = a.tile_y;
    load_member(&M, a.members + t.member);
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();
    const int nl = M.nl;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        const bool ring = on_ring(j, i, M.Ny, M.Nx);
        const bool land = is_land(M, j, i);  // q reads as zero on land
        float v[kMaxLayers];
        for (int l = 0; l < nl; ++l) {
            const float x = a.q[caller_idx(M, l, j, i)];
            if (a.copy) a.copy[xrow_idx(M, l, j, i)] = (a.zero_ring_copy && (ring || land)) ? 0.f : x;
            v[l] = ((a.bc_operand && ring) || land) ? 0.f : x;
        }
        if (!a.xa) continue;
        for (int m = 0; m < nl; ++m) {
            float s = 0.f;
            for (int l = 0; l < nl; ++l) s = fmaf(M.Cl2m[m * kMaxLayers + l], v[l], s);
            store_plane(a.xa, a.xa_fmt, a.xplane, xrow_idx(M, m, j, i), s);
            if (a.xq) a.xq[xrow_idx(M, m, j, i)] = s;
        }
    }
}

// Unpack: internal plane -> caller packing (every cell, ring included).
__global__ void __launch_bounds__(NTHREADS) k_unpack(const MemberDev* __restrict__ members,
                                                     const StencilTile* __restrict__ tiles, int TX, int TY,
                                                     const float* __restrict__ src, float* __restrict__ q) {
    __shared__ MemberDev M;
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        for (int l = 0; l < M.nl; ++l) q[caller_idx(M, l, j, i)] = src[xrow_idx(M, l, j, i)];
    }
}

// ---------------------------------------------------------------------------------------
// Butcher-form stage combine (Euler, Tsit5): out = y0 + dt * sum_j c_j k_j over the stage
// derivatives k_j (caller packing, one plane of `kplane` floats each), into an x-row stage
// plane, plus the modal operand of that stage input (BC: zero ring and land) for the next DST
// solve.  The ring is combined like every other cell; stage inputs are read with the BC, and
// the final combination's ring is y0 + dt * wind as in the fused Shu-Osher stencil.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_rk_combine(RkCombineArgs a) {
    __shared__ MemberDev M;
    const StencilTile t = a.tiles[blockIdx.x];
    load_member(&M, a.members + t.member);
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();
    const int nl = M.nl, TX = a.tile_x, TY = a.tile_y;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        const bool zero = on_ring(j, i, M.Ny, M.Nx) || is_land(M, j, i);
        float v[kMaxLayers];
        for (int l = 0; l < nl; ++l) {
            const int64_t ci = caller_idx(M, l, j, i);
            float acc = 0.f;
            for (int s = 0; s < a.n_k; ++s)
                if (a.coef[s] != 0.f) acc = fmaf(a.coef[s], a.k[(int64_t)s * a.kplane + ci], acc);
            const int64_t xi = xrow_idx(M, l, j, i);
            v[l] = a.y0[xi] + a.dt * acc;
            a.out[xi] = v[l];
        }
        for (int m = 0; m < nl; ++m) {
            float sum = 0.f;
            if (!zero)
                for (int l = 0; l < nl; ++l) sum = fmaf(M.Cl2m[m * kMaxLayers + l], v[l], sum);
            store_plane(a.xa, a.xa_fmt, a.xplane, xrow_idx(M, m, j, i), sum);
            if (a.xq) a.xq[xrow_idx(M, m, j, i)] = sum;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Mode -> layer epilogue for qg_invert: psi = Cm2l psi_hat, ring zeroed (baroclinic).
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_mode_to_layer(const MemberDev* __restrict__ members,
                                                            const StencilTile* __restrict__ tiles, int TX, int TY,
                                                            const float* __restrict__ psi_hat,
                                                            float* __restrict__ psi) {
    __shared__ MemberDev M;
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();
    const int nl = M.nl;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        const bool zero = (!M.barotropic && on_ring(j, i, M.Ny, M.Nx)) || is_land(M, j, i);
        float ph[kMaxLayers];
        for (int m = 0; m < nl; ++m) ph[m] = psi_hat[xrow_idx(M, m, j, i)];
        for (int l = 0; l < nl; ++l) {
            float p = 0.f;
            for (int m = 0; m < nl; ++m) p = fmaf(M.Cm2l[l * kMaxLayers + m], ph[m], p);
            psi[caller_idx(M, l, j, i)] = zero ? 0.f : p;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Geostrophic projection of a multilayer shallow-water state (h, u, v) around one modal
// Helmholtz inversion (ReparameterizedQG.project, reparameterized.py:142-178), all fields in
// the caller's packing on the Arakawa C-grid of the arrays (u at the east faces, v at the
// north faces, vorticity and the streamfunction's corner points at index (j, i) of the
// north-east corner of T-cell (j, i)):
//   k_project_q: q = zeta - f0 (h - H_l) / H_l with zeta = (v[j][i+1] - v[j][i]) / dx
//                - (u[j+1][i] - u[j][i]) / dy on interior cells, 0 on the ring
//   k_project_g: u_g = -(psi[j][i] - psi[j-1][i]) / dy, v_g = (psi[j][i] - psi[j][i-1]) / dx
//                on interior cells (0 on the ring), h_g = H_l (1 + f0 (Cm2l diag(eig) Cl2m
//                psi)_l) with eig_m = lambda_m / f0^2 everywhere
// The curl of grad_perp is then the 5-point Laplacian, so Q G is the Helmholtz operator the
// inversion solves and the projection is idempotent up to the ring.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_project_q(const MemberDev* __restrict__ members,
                                                        const StencilTile* __restrict__ tiles, int TX, int TY,
                                                        const float* __restrict__ h, const float* __restrict__ u,
                                                        const float* __restrict__ v, float* __restrict__ q) {
    __shared__ MemberDev M;
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();
    const float idx = 1.f / M.dx, idy = 1.f / M.dy;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        const bool ring = on_ring(j, i, M.Ny, M.Nx);
        for (int l = 0; l < M.nl; ++l) {
            const int64_t o = caller_idx(M, l, j, i);
            float zeta = 0.f;
            if (!ring) zeta = (v[o + 1] - v[o]) * idx - (u[o + M.Nx] - u[o]) * idy;
            q[o] = zeta - M.f0 * ((h[o] - M.H[l]) / M.H[l]);
        }
    }
}

__global__ void __launch_bounds__(NTHREADS) k_project_g(const MemberDev* __restrict__ members,
                                                        const StencilTile* __restrict__ tiles, int TX, int TY,
                                                        const float* __restrict__ psi, float* __restrict__ hg,
                                                        float* __restrict__ ug, float* __restrict__ vg) {
    __shared__ MemberDev M;
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();
    const int nl = M.nl;
    const float idx = 1.f / M.dx, idy = 1.f / M.dy, if0 = 1.f / M.f0;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        const bool ring = on_ring(j, i, M.Ny, M.Nx);
        float p[kMaxLayers], pm[kMaxLayers];
        for (int l = 0; l < nl; ++l) p[l] = psi[caller_idx(M, l, j, i)];
        for (int m = 0; m < nl; ++m) {
            float s = 0.f;
            for (int k = 0; k < nl; ++k) s = fmaf(M.Cl2m[m * kMaxLayers + k], p[k], s);
            pm[m] = s * (M.lam[m] * if0);  // f0 eig_m (Cl2m psi)_m
        }
        for (int l = 0; l < nl; ++l) {
            const int64_t o = caller_idx(M, l, j, i);
            float a = 0.f;
            for (int m = 0; m < nl; ++m) a = fmaf(M.Cm2l[l * kMaxLayers + m], pm[m], a);
            hg[o] = fmaf(M.H[l], a, M.H[l]);  // H + H a: the anomaly rounds once
            ug[o] = ring ? 0.f : -(p[l] - psi[o - M.Nx]) * idy;
            vg[o] = ring ? 0.f : (p[l] - psi[o - 1]) * idx;
        }
    }
}

// The transposes of the two projection kernels (the reverse mode of ReparameterizedQG.project):
//   k_project_g_vjp: psi_bar = G^T (h_g_bar, u_g_bar, v_g_bar): per cell Cl2m^T diag(f0 eig)
//                    Cm2l^T (H h_g_bar), plus the transposed grad_perp differences
//   k_project_q_vjp: (h_bar, u_bar, v_bar) = Q^T q_bar: h_bar = -f0 q_bar / H_l, the transposed
//                    curl differences for u_bar and v_bar
__global__ void __launch_bounds__(NTHREADS) k_project_g_vjp(const MemberDev* __restrict__ members,
                                                            const StencilTile* __restrict__ tiles, int TX, int TY,
                                                            const float* __restrict__ hgb, const float* __restrict__ ugb,
                                                            const float* __restrict__ vgb, float* __restrict__ psib) {
    __shared__ MemberDev M;
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    const int nl = M.nl;
    const float idx = 1.f / M.dx, idy = 1.f / M.dy, if0 = 1.f / M.f0;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        auto interior = [&](int a, int b) { return a >= 1 && a <= M.Ny - 2 && b >= 1 && b <= M.Nx - 2; };
        float w[kMaxLayers], wm[kMaxLayers];
        for (int l = 0; l < nl; ++l) w[l] = M.H[l] * hgb[caller_idx(M, l, j, i)];
        for (int m = 0; m < nl; ++m) {  // (Cm2l^T w)_m scaled by f0 eig_m
            float s = 0.f;
            for (int l = 0; l < nl; ++l) s = fmaf(M.Cm2l[l * kMaxLayers + m], w[l], s);
            wm[m] = s * (M.lam[m] * if0);
        }
        for (int k = 0; k < nl; ++k) {
            float s = 0.f;
            for (int m = 0; m < nl; ++m) s = fmaf(M.Cl2m[m * kMaxLayers + k], wm[m], s);
            const int64_t o = caller_idx(M, k, j, i);
            // u_g(a, b) = -(psi(a, b) - psi(a - 1, b)) / dy, v_g(a, b) = (psi(a, b) - psi(a, b - 1)) / dx
            if (interior(j, i)) s += -ugb[o] * idy + vgb[o] * idx;
            if (interior(j + 1, i)) s += ugb[o + M.Nx] * idy;
            if (interior(j, i + 1)) s -= vgb[o + 1] * idx;
            psib[o] = s;
        }
    }
}

__global__ void __launch_bounds__(NTHREADS) k_project_q_vjp(const MemberDev* __restrict__ members,
                                                            const StencilTile* __restrict__ tiles, int TX, int TY,
                                                            const float* __restrict__ qb, float* __restrict__ hb,
                                                            float* __restrict__ ub, float* __restrict__ vb) {
    __shared__ MemberDev M;
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    const float idx = 1.f / M.dx, idy = 1.f / M.dy;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= M.Ny || i >= M.Nx) continue;
        auto interior = [&](int a, int b) { return a >= 1 && a <= M.Ny - 2 && b >= 1 && b <= M.Nx - 2; };
        for (int l = 0; l < M.nl; ++l) {
            const int64_t o = caller_idx(M, l, j, i);
            // zeta(a, b) = (v(a, b + 1) - v(a, b)) / dx - (u(a + 1, b) - u(a, b)) / dy
            float u = 0.f, v = 0.f;
            if (interior(j, i)) {
                u += qb[o] * idy;
                v -= qb[o] * idx;
            }
            if (interior(j - 1, i)) u -= qb[o - M.Nx] * idy;
            if (interior(j, i - 1)) v += qb[o - 1] * idx;
            hb[o] = -M.f0 * qb[o] / M.H[l];
            ub[o] = u;
            vb[o] = v;
        }
    }
}

// ---------------------------------------------------------------------------------------
// Helmholtz residual in modal space for one refinement sweep:
//   r_m = qm_m - (lap_full psi_hat_m - lam_m psi_hat_m)
// where lap_full is the full-array 5-point operator with zeros outside the array (the
// operator the DST-I solve inverts).  qm is the FP32 modal right-hand side.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_residual(const MemberDev* __restrict__ members,
                                                       const StencilTile* __restrict__ tiles, int TX, int TY,
                                                       const float* __restrict__ qm,
                                                       const float* __restrict__ psi_hat,
                                                       void* out, int out_fmt, int64_t xplane) {
    __shared__ MemberDev M;
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();
    const int nl = M.nl, Ny = M.Ny, Nx = M.Nx;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= Ny || i >= Nx) continue;
        for (int m = 0; m < nl; ++m) {
            auto P = [&](int jj, int ii) {
                return (jj < 0 || jj >= Ny || ii < 0 || ii >= Nx) ? 0.f : psi_hat[xrow_idx(M, m, jj, ii)];
            };
            const float c0 = P(j, i);
            const float lap = (P(j, i + 1) - 2.f * c0 + P(j, i - 1)) * M.inv_dx2 +
                              (P(j + 1, i) - 2.f * c0 + P(j - 1, i)) * M.inv_dy2;
            const float r = qm[xrow_idx(M, m, j, i)] - (lap - M.lam[m] * c0);
            store_plane(out, out_fmt, xplane, xrow_idx(M, m, j, i), r);
        }
    }
}

// ---------------------------------------------------------------------------------------
// Diagnostics (baroclinic.py:197-228): per layer KE = 1/2 sum_int (u_T^2 + v_T^2) dx dy,
// enstrophy = 1/2 sum_int q^2 dx dy, u = -d_y psi (V points), v = d_x psi (U points),
// both interior-written and averaged back to T points.  Sums accumulate in double.
// ---------------------------------------------------------------------------------------
__global__ void __launch_bounds__(NTHREADS) k_diag(const MemberDev* __restrict__ members,
                                                   const StencilTile* __restrict__ tiles, int TX, int TY,
                                                   const float* __restrict__ q,
                                                   const float* __restrict__ psi_hat,
                                                   double* __restrict__ acc) {
    __shared__ MemberDev M;
    __shared__ double red[2 * kMaxLayers][NTHREADS / 32];
    const StencilTile t = tiles[blockIdx.x];
    load_member(&M, members + t.member);
    __syncthreads();
    pdl_wait();
    pdl_launch_dependents();
    const int nl = M.nl, Ny = M.Ny, Nx = M.Nx;
    double ke[kMaxLayers], en[kMaxLayers];
    for (int l = 0; l < nl; ++l) ke[l] = en[l] = 0.0;
    auto psi = [&](int l, int j, int i) -> float {
        if (j <= 0 || i <= 0 || j >= Ny - 1 || i >= Nx - 1) {
            if (!M.barotropic || j < 0 || i < 0 || j >= Ny || i >= Nx) return 0.f;
        }
        if (is_land(M, j, i)) return 0.f;
        float p = 0.f;
        for (int m = 0; m < nl; ++m) p = fmaf(M.Cm2l[l * kMaxLayers + m], psi_hat[xrow_idx(M, m, j, i)], p);
        return p;
    };
    auto uV = [&](int l, int j, int i) -> float {
        if (j <= 0 || i <= 0 || j >= Ny - 1 || i >= Nx - 1) return 0.f;
        return -(psi(l, j + 1, i) - psi(l, j, i)) / M.dy;
    };
    auto vU = [&](int l, int j, int i) -> float {
        if (j <= 0 || i <= 0 || j >= Ny - 1 || i >= Nx - 1) return 0.f;
        return (psi(l, j, i + 1) - psi(l, j, i)) / M.dx;
    };
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j <= 0 || i <= 0 || j >= Ny - 1 || i >= Nx - 1) continue;
        for (int l = 0; l < nl; ++l) {
            const float uT = 0.5f * (uV(l, j, i) + uV(l, j - 1, i));
            const float vT = 0.5f * (vU(l, j, i) + vU(l, j, i - 1));
            ke[l] += (double)uT * uT + (double)vT * vT;
            const float qv = is_land(M, j, i) ? 0.f : q[caller_idx(M, l, j, i)];
            en[l] += (double)qv * qv;
        }
    }
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int l = 0; l < nl; ++l) {
        double x = ke[l], y = en[l];
        for (int o = 16; o > 0; o >>= 1) {
            x += __shfl_down_sync(0xffffffffu, x, o);
            y += __shfl_down_sync(0xffffffffu, y, o);
        }
        if (lane == 0) {
            red[l][w] = x;
            red[kMaxLayers + l][w] = y;
        }
    }
    __syncthreads();
    if (threadIdx.x < nl) {
        const int l = threadIdx.x;
        double x = 0.0, y = 0.0;
        for (int k = 0; k < NTHREADS / 32; ++k) {
            x += red[l][k];
            y += red[kMaxLayers + l][k];
        }
        const double area = 0.5 * (double)M.dx * (double)M.dy;
        atomicAdd(&acc[2 * (M.off_layer + l)], x * area);
        atomicAdd(&acc[2 * (M.off_layer + l) + 1], y * area);
    }
}

// The velocity and vorticity fields of diagnose (baroclinic.py:197-228) from the layer psi
// (caller packing): u = -d_y psi on the V points, v = d_x psi on the U points (forward
// differences written to the interior), zeta = lap(psi) (5-point, interior); the ring is 0.
__global__ void __launch_bounds__(NTHREADS) k_diag_fields(const MemberDev* __restrict__ members,
                                                          const StencilTile* __restrict__ tiles, int TX, int TY,
                                                          const float* __restrict__ psi, float* __restrict__ u,
                                                          float* __restrict__ v, float* __restrict__ zeta) {
    const StencilTile t = tiles[blockIdx.x];
    const MemberDev& M = members[t.member];
    const int nl = M.nl, Ny = M.Ny, Nx = M.Nx;
    const float idx = 1.f / M.dx, idy = 1.f / M.dy, idx2 = M.inv_dx2, idy2 = M.inv_dy2;
    for (int c = threadIdx.x; c < TX * TY; c += blockDim.x) {
        const int j = t.ty * TY + c / TX, i = t.tx * TX + c % TX;
        if (j >= Ny || i >= Nx) continue;
        const bool in = j > 0 && i > 0 && j < Ny - 1 && i < Nx - 1;
        for (int l = 0; l < nl; ++l) {
            const int64_t o = caller_idx(M, l, j, i);
            float uu = 0.f, vv = 0.f, zz = 0.f;
            if (in) {
                const float pc = psi[o], pn = psi[o + Nx], ps = psi[o - Nx], pe = psi[o + 1], pw = psi[o - 1];
                uu = -(pn - pc) * idy;
                vv = (pe - pc) * idx;
                zz = (pe - 2.f * pc + pw) * idx2 + (pn - 2.f * pc + ps) * idy2;
            }
            u[o] = uu;
            v[o] = vv;
            zeta[o] = zz;
        }
    }
}

cudaError_t launch_diag_fields(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                               const float* psi, float* u, float* v, float* zeta, cudaStream_t s) {
    return launch_k(k_diag_fields, ntiles, NTHREADS, 0, s, false, members, tiles, large ? TileL::TX : TileS::TX,
                    large ? TileL::TY : TileS::TY, psi, u, v, zeta);
}

__global__ void k_diag_finish(const double* __restrict__ acc, int64_t n, float* ke, float* ens) {
    pdl_wait();
    pdl_launch_dependents();
    const int64_t l = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (l < n) {
        ke[l] = (float)acc[2 * l];
        ens[l] = (float)acc[2 * l + 1];
    }
}

// ---------------------------------------------------------------------------------------
// State statistics of the runner: min / mean / max over the finite entries of a packed
// field and the count of non-finite ones, reduced on the device (one atomic per block).
// acc: [0] min and [1] max as order-preserving ints, [2] the finite sum (double, in acc_d),
// [3] finite and [4] non-finite counts.
// ---------------------------------------------------------------------------------------
__device__ __forceinline__ int ordered_int(float f) {
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7fffffff;
}
__device__ __forceinline__ float from_ordered(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7fffffff); }

struct StatsAcc {
    int mn, mx;
    double sum;
    unsigned long long n_finite, n_bad;
};

__global__ void k_stats_init(StatsAcc* acc) {
    acc->mn = ordered_int(INFINITY);
    acc->mx = ordered_int(-INFINITY);
    acc->sum = 0.0;
    acc->n_finite = acc->n_bad = 0ull;
}

__global__ void __launch_bounds__(256) k_stats(const float* __restrict__ q, int64_t n, StatsAcc* acc) {
    float mn = INFINITY, mx = -INFINITY;
    double sum = 0.0;
    unsigned long long nf = 0, nb = 0;
    auto take = [&](float v) {
        if (isfinite(v)) {
            mn = fminf(mn, v);
            mx = fmaxf(mx, v);
            sum += (double)v;
            ++nf;
        } else {
            ++nb;
        }
    };
    const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    const int64_t nth = (int64_t)gridDim.x * blockDim.x;
    const bool vec = (reinterpret_cast<uintptr_t>(q) & 15) == 0;
    const int64_t n4 = vec ? n / 4 : 0;
    for (int64_t i = tid; i < n4; i += nth) {
        const float4 v = __ldg(reinterpret_cast<const float4*>(q) + i);
        take(v.x);
        take(v.y);
        take(v.z);
        take(v.w);
    }
    for (int64_t i = 4 * n4 + tid; i < n; i += nth) take(q[i]);
    for (int o = 16; o > 0; o >>= 1) {
        mn = fminf(mn, __shfl_xor_sync(0xffffffffu, mn, o));
        mx = fmaxf(mx, __shfl_xor_sync(0xffffffffu, mx, o));
        sum += __shfl_xor_sync(0xffffffffu, sum, o);
        nf += __shfl_xor_sync(0xffffffffu, nf, o);
        nb += __shfl_xor_sync(0xffffffffu, nb, o);
    }
    __shared__ StatsAcc part[8];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) part[w] = {ordered_int(mn), ordered_int(mx), sum, nf, nb};
    __syncthreads();
    if (threadIdx.x == 0) {
        StatsAcc b = part[0];
        for (int k = 1; k < (int)(blockDim.x >> 5); ++k) {
            b.mn = min(b.mn, part[k].mn);
            b.mx = max(b.mx, part[k].mx);
            b.sum += part[k].sum;
            b.n_finite += part[k].n_finite;
            b.n_bad += part[k].n_bad;
        }
        atomicMin(&acc->mn, b.mn);
        atomicMax(&acc->mx, b.mx);
        atomicAdd(&acc->sum, b.sum);
        atomicAdd(&acc->n_finite, b.n_finite);
        atomicAdd(&acc->n_bad, b.n_bad);
    }
}

__global__ void k_stats_finish(const StatsAcc* acc, double* out) {
    const bool any = acc->n_finite > 0;
    out[0] = any ? (double)from_ordered(acc->mn) : NAN;
    out[1] = any ? acc->sum / (double)acc->n_finite : NAN;
    out[2] = any ? (double)from_ordered(acc->mx) : NAN;
    out[3] = (double)acc->n_bad;
}

cudaError_t launch_state_stats(const float* q, int64_t n, void* acc, double* out, int grid, cudaStream_t s) {
    StatsAcc* a = static_cast<StatsAcc*>(acc);
    cudaError_t e = launch_k(k_stats_init, 1, 1, 0, s, false, a);
    if (!e) e = launch_k(k_stats, grid, 256, 0, s, false, q, n, a);
    if (!e) e = launch_k(k_stats_finish, 1, 1, 0, s, false, (const StatsAcc*)a, out);
    return e;
}

// ---------------------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------------------
// 3-D boxes (BX, BY, nl) over a member's x-row planes: dims (Nx, Ny, nl), row pitch Px.
cudaError_t stencil_encode_maps(const MemberDev& M, const float* const planes[4], int large, void* out) {
    StencilMaps sm;
    memset(&sm, 0, sizeof(sm));
    const uint64_t dims[3] = {(uint64_t)M.Nx, (uint64_t)M.Ny, (uint64_t)M.nl};
    const uint64_t strides[2] = {(uint64_t)M.Px * 4, (uint64_t)M.Px * M.Ny * 4};
    const uint32_t box[3] = {(uint32_t)(large ? TileL::BX : TileS::BX), (uint32_t)(large ? TileL::BY : TileS::BY),
                             (uint32_t)M.nl};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 4 && !e; ++k) {
        CUtensorMap* m = k < 3 ? &sm.q[k] : &sm.psi;
        e = tmap_encode(m, 0, 3, planes[k] + M.off_x, dims, strides, box, 0);
    }
    if (!e) memcpy(out, &sm, sizeof(sm));
    return e;
}

cudaError_t launch_prep(const PrepArgs& a, int ntiles, cudaStream_t s, bool pdl) {
    return launch_k(k_prep, ntiles, NTHREADS, 0, s, pdl, a);
}

cudaError_t launch_rk_combine(const RkCombineArgs& a, int ntiles, cudaStream_t s, bool pdl) {
    return launch_k(k_rk_combine, ntiles, NTHREADS, 0, s, pdl, a);
}

cudaError_t launch_unpack(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                          const float* src, float* q, cudaStream_t s, bool pdl) {
    return launch_k(k_unpack, ntiles, NTHREADS, 0, s, pdl, members, tiles, large ? TileL::TX : TileS::TX,
                    large ? TileL::TY : TileS::TY, src, q);
}

cudaError_t launch_mode_to_layer(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                                 const float* psi_hat, float* psi, cudaStream_t s, bool pdl) {
    return launch_k(k_mode_to_layer, ntiles, NTHREADS, 0, s, pdl, members, tiles, large ? TileL::TX : TileS::TX,
                    large ? TileL::TY : TileS::TY, psi_hat, psi);
}

cudaError_t launch_project_q(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                             const float* h, const float* u, const float* v, float* q, cudaStream_t s) {
    return launch_k(k_project_q, ntiles, NTHREADS, 0, s, false, members, tiles, large ? TileL::TX : TileS::TX,
                    large ? TileL::TY : TileS::TY, h, u, v, q);
}

cudaError_t launch_project_g(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                             const float* psi, float* hg, float* ug, float* vg, cudaStream_t s) {
    return launch_k(k_project_g, ntiles, NTHREADS, 0, s, false, members, tiles, large ? TileL::TX : TileS::TX,
                    large ? TileL::TY : TileS::TY, psi, hg, ug, vg);
}

cudaError_t launch_project_g_vjp(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                                 const float* hgb, const float* ugb, const float* vgb, float* psib, cudaStream_t s) {
    return launch_k(k_project_g_vjp, ntiles, NTHREADS, 0, s, false, members, tiles, large ? TileL::TX : TileS::TX,
                    large ? TileL::TY : TileS::TY, hgb, ugb, vgb, psib);
}

cudaError_t launch_project_q_vjp(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                                 const float* qb, float* hb, float* ub, float* vb, cudaStream_t s) {
    return launch_k(k_project_q_vjp, ntiles, NTHREADS, 0, s, false, members, tiles, large ? TileL::TX : TileS::TX,
                    large ? TileL::TY : TileS::TY, qb, hb, ub, vb);
}

cudaError_t launch_residual(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                            const float* qm, const float* psi_hat, void* out, int out_fmt,
                            int64_t xplane, cudaStream_t s, bool pdl) {
    return launch_k(k_residual, ntiles, NTHREADS, 0, s, pdl, members, tiles, large ? TileL::TX : TileS::TX,
                    large ? TileL::TY : TileS::TY, qm, psi_hat, out, out_fmt, xplane);
}

cudaError_t launch_diag_acc(const MemberDev* members, const StencilTile* tiles, int ntiles, int large,
                            const float* q, const float* psi_hat, double* acc, cudaStream_t s) {
    return launch_k(k_diag, ntiles, NTHREADS, 0, s, false, members, tiles, large ? TileL::TX : TileS::TX,
                    large ? TileL::TY : TileS::TY, q, psi_hat, acc);
}

cudaError_t launch_diag_finish(const double* acc, int64_t n_layers, float* ke, float* ens,
                               cudaStream_t s) {
    return launch_k(k_diag_finish, (int)((n_layers + 127) / 128), 128, 0, s, false, acc, n_layers, ke, ens);
}

}  // namespace qg
