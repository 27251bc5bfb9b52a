// Cluster-resident time stepping of small members (the latency-bound regime).
//
// One thread-block cluster of C CTAs (one per SM) holds a member for a whole qg_step call:
// every stage of every step runs in one launch, the state and all intermediate planes stay
// in shared memory, and the phases meet at hardware cluster barriers instead of kernel
// boundaries.  The member is cut into C row blocks along y and C column blocks along x; CTA c
// owns y in [c By, c By + By) and x in [c Bx, c Bx + Bx).
//
// The DST-I inversion is four FP32 passes on the CUDA cores, each contracting one axis of
// the CTA's own rows against the orthonormal DST-I matrix S (symmetric, S S = I) held in
// shared memory.  S is folded: S[K-1-k][n] = (-1)^n S[k][n], so out[n] = sum over k < K/2 of
// (in[k] + in[K-1-k]) S[k][n] for even n and of (in[k] - in[K-1-k]) S[k][n] for odd n, half
// the multiply-adds of the dense product.  A pass's result goes to the CTAs that own its
// output index (the transpose between passes), staged in local shared memory and pushed as
// 16-byte stores into the owners' shared memory (distributed shared memory), then one
// cluster barrier.  Pass order and operands follow the multi-launch path: G1 contracts x,
// G2 y (and divides by ex + ey - lambda), G3 x, G4 y; G4 also fills the one-row y halos of
// its owners.  The stencil (the same arithmetic as the column-sweep and tile stencils, one
// thread per cell and all layers, so that the Cl2m operand of the next stage is formed in
// place) updates the stage, writes the next stage input with its two-row y halos into the
// neighbouring CTAs, and forms the next operand for G1 in the CTA's own rows.
//
// Every plane uses one layout, [layer][k][b]: k the full index the next pass contracts (or
// x for the stencil's planes), b the CTA's local index (y or x) padded to a multiple of 4.
#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {

namespace {

constexpr int kClThreads = 384;

__device__ __forceinline__ unsigned cl_rank() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}
__device__ __forceinline__ unsigned cl_size() {
    unsigned r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}
// All threads of every CTA of the cluster; orders shared (local and remote) and global
// memory at cluster scope.
__device__ __forceinline__ void cl_sync() {
    asm volatile(
        "barrier.cluster.arrive.release.aligned;\n"
        "barrier.cluster.wait.acquire.aligned;" ::
            : "memory");
}
// The shared::cluster address of `p` (a location of this CTA's shared memory) in CTA `rank`.
__device__ __forceinline__ uint32_t cl_map(const void* p, unsigned rank) {
    uint32_t r;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(r) : "r"(su32(p)), "r"(rank));
    return r;
}
// Remote stores carry no memory clobber (they only read registers); the cluster barrier's
// clobber and the order of volatile asm keep them before the barrier that publishes them.
__device__ __forceinline__ void cl_st4(uint32_t a, float4 v) {
    asm volatile("st.shared::cluster.v4.f32 [%0], {%1, %2, %3, %4};" ::"r"(a), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w));
}
__device__ __forceinline__ void cl_st(uint32_t a, float v) {
    asm volatile("st.shared::cluster.f32 [%0], %1;" ::"r"(a), "f"(v));
}

__device__ __forceinline__ bool ring_cell(int y, int x, int Ny, int Nx) {
    return y == 0 || x == 0 || y == Ny - 1 || x == Nx - 1;
}

// Per-member scalars, held in registers for the whole launch.
struct ClConst {
    int Ny, Nx, barotropic;
    float idx2, idy2, i12, b12;
    float nu, kappa, nu4, wind_s;  // wind_s = tau0 / H0 (top layer)
};

// Per-member tables copied into shared memory at the start (at g.o_const): Cm2l [NL][NL]
// (psi of layer l from mode m at l * NL + m), Cl2m [NL][NL] (mode m from layer l at m * NL + l),
// lambda [NL], the wind profile F [Ny], the DST-I eigenvalues ex [Nx] and ey [Ny].
template <int NL>
struct ClTables {
    const float *cm, *cl, *lam, *F, *ex, *ey;
};
template <int NL>
__device__ __forceinline__ ClTables<NL> cl_tables(const float* sm, const ClGeom& g, int Ny, int Nx) {
    ClTables<NL> t;
    t.cm = sm + g.o_const;
    t.cl = t.cm + NL * NL;
    t.lam = t.cl + NL * NL;
    t.F = t.lam + NL;
    t.ex = t.F + Ny;
    t.ey = t.ex + Nx;
    return t;
}

struct ClusterArgs {
    const MemberDev* members;
    float* q;             // caller packing, in / out
    const float* params;  // n_members * QG_NPARAMS
    int apply_bc;         // zero the ring of the state first
    int n_steps, n_stages;
    float sa[4], sb[4], dt;
    int* flags;
};

// One DST-I pass on this CTA's rows (see the file comment).  in: [NL][K][BPin] with Bc valid
// local rows; the result for output index n goes to owner o = n / Bn, into its buffer at
// float offset dst ([NL][Ktot][BPo]), row b0 + b, column n - o Bn (+ 1 with HALO, which also
// copies the first and last index of each block into the neighbouring blocks' halos).
// DIV: divide by ex[b0 + b] + ey[n] - lambda_l (G2).
template <int NL, bool DIV, bool HALO>
__device__ void dst_pass(float* sm, const ClGeom& g, const ClTables<NL>& T, const float* in, int K, int Bc, int BPin,
                         const float* Sh, int NP, int b0, int Ktot, int Bn, int BPo, int dst) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int H = (K + 1) / 2;
    float* fold = sm + g.o_fold;  // [NL][H][2][BPin]
    float* stg = sm + g.o_stg;    // [owner][NL][Bc][BPo]
    const int C = g.C;
    if (Bc > 0) {
        for (int i = tid; i < NL * H * BPin; i += nt) {
            const int b = i % BPin, lk = i / BPin, k = lk % H, l = lk / H;
            const float lo = in[(l * K + k) * BPin + b];
            const int kk = K - 1 - k;
            const float hi = kk != k ? in[(l * K + kk) * BPin + b] : 0.f;
            fold[(lk * 2) * BPin + b] = lo + hi;
            fold[(lk * 2 + 1) * BPin + b] = kk != k ? lo - hi : 0.f;
        }
        __syncthreads();
        const int nbq = (Bc + 3) / 4, nnq = NP / 4;
        for (int t = tid; t < NL * nbq * nnq; t += nt) {
            const int nq = t % nnq, lb = t / nnq, bq = lb % nbq, l = lb / nbq;
            float acc[4][4];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;
            const float* f = fold + (l * H * 2) * BPin + bq * 4;
            const float* s = Sh + nq * 4;
#pragma unroll 4
            for (int k = 0; k < H; ++k) {
                const float4 ev = *reinterpret_cast<const float4*>(f + (2 * k) * BPin);
                const float4 od = *reinterpret_cast<const float4*>(f + (2 * k + 1) * BPin);
                const float4 sv = *reinterpret_cast<const float4*>(s + k * NP);
                const float e4[4] = {ev.x, ev.y, ev.z, ev.w}, o4[4] = {od.x, od.y, od.z, od.w};
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    acc[i][0] = fmaf(e4[i], sv.x, acc[i][0]);
                    acc[i][1] = fmaf(o4[i], sv.y, acc[i][1]);
                    acc[i][2] = fmaf(e4[i], sv.z, acc[i][2]);
                    acc[i][3] = fmaf(o4[i], sv.w, acc[i][3]);
                }
            }
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int b = bq * 4 + i;
                if (b >= Bc) continue;
#pragma unroll
                for (int j = 0; j < 4; ++j) {
                    const int n = nq * 4 + j;
                    if (n >= K) continue;
                    float v = acc[i][j];
                    if (DIV) v = v / (T.ex[b0 + b] + T.ey[n] - T.lam[l]);
                    const int o = n / Bn, cn = n - o * Bn;
                    stg[((o * NL + l) * Bc + b) * BPo + cn + (HALO ? 1 : 0)] = v;
                    if (HALO) {
                        if (cn == 0 && o > 0) stg[(((o - 1) * NL + l) * Bc + b) * BPo + Bn + 1] = v;
                        if (cn == Bn - 1 && o + 1 < C) stg[(((o + 1) * NL + l) * Bc + b) * BPo] = v;
                    }
                }
            }
        }
        __syncthreads();
        // push the owners' chunks: rows b0 .. b0 + Bc of each layer are contiguous there
        const int per = Bc * BPo / 4;  // float4 per (owner, layer)
        for (int i = tid; i < C * NL * per; i += nt) {
            const int f4 = i % per, ol = i / per, l = ol % NL, o = ol / NL;
            if (o * Bn >= K) continue;  // empty block
            const float4 v = *reinterpret_cast<const float4*>(stg + (size_t)ol * Bc * BPo + f4 * 4);
            cl_st4(cl_map(sm + dst + (l * Ktot + b0) * BPo + f4 * 4, o), v);
        }
    }
}

// The stage's stencil on this CTA's rows y0 .. y0 + Bc (see the file comment); qs: stage input
// [NL][Nx][BPq] (rows y0 - 2 ..), qn: next stage input, same layout, in every CTA.
template <int NL>
__device__ void cl_stencil(float* sm, const ClGeom& g, const ClConst& K, const ClTables<NL>& T, int c, int y0,
                           int Bc, int qs_off, int qn_off, float sa, float sb, float dt, bool fin, bool& bad) {
    const int tid = threadIdx.x, nt = blockDim.x;
    const int Ny = K.Ny, Nx = K.Nx;
    const int BPe = g.BPe, BPq = g.BPq, BPy = g.BPy;
    float* psi = sm + g.o_psi;   // [NL][Nx][BPe]: modes of psi_hat in, layers of psi out
    float* lq = sm + g.o_fold;   // [NL][Nx][BPe]: lap q
    const float* qs = sm + qs_off;
    float* y0b = sm + g.o_y0;    // [NL][Nx][BPy]
    float* op = sm + g.o_rb;     // next operand, [NL][Nx][BPy]
    const bool zero_psi_ring = !K.barotropic;
    const float i12 = K.i12, b12 = K.b12, idx2 = K.idx2, idy2 = K.idy2;
    if (Bc > 0) {
        for (int i = tid; i < Nx * (Bc + 2); i += nt) {
            const int be = i % (Bc + 2), x = i / (Bc + 2), y = y0 - 1 + be;
            const bool in = y >= 0 && y < Ny;
            float h[NL];
#pragma unroll
            for (int m = 0; m < NL; ++m) h[m] = in ? psi[(m * Nx + x) * BPe + be] : 0.f;
            const bool zr = !in || (zero_psi_ring && ring_cell(y, x, Ny, Nx));
#pragma unroll
            for (int l = 0; l < NL; ++l) {
                float v = 0.f;
#pragma unroll
                for (int m = 0; m < NL; ++m) v = fmaf(T.cm[l * NL + m], h[m], v);
                psi[(l * Nx + x) * BPe + be] = zr ? 0.f : v;
            }
            // lap q (zero on the ring and outside)
            const bool lin = in && !ring_cell(y, x, Ny, Nx);
#pragma unroll
            for (int l = 0; l < NL; ++l) {
                float v = 0.f;
                if (lin) {
                    const float* qc = qs + (l * Nx + x) * BPq + be + 1;
                    const float c0 = qc[0];
                    v = (qc[BPq] + qc[-BPq] - 2.f * c0) * idx2 + (qc[1] + qc[-1] - 2.f * c0) * idy2;
                }
                lq[(l * Nx + x) * BPe + be] = v;
            }
        }
        __syncthreads();
        const float nu = K.nu, kappa = K.kappa, nu4 = K.nu4, wind_s = K.wind_s;
        const unsigned up = c > 0 ? (unsigned)c - 1 : 0u, down = (unsigned)c + 1;
        const bool has_up = c > 0, has_down = (int)down < g.C;
        for (int i = tid; i < Nx * Bc; i += nt) {
            const int b = i % Bc, x = i / Bc, y = y0 + b;
            const bool ring = ring_cell(y, x, Ny, Nx);
            const float wr = wind_s * T.F[y];
            float yn[NL];
#pragma unroll
            for (int l = 0; l < NL; ++l) {
                const float* f = psi + (l * Nx + x) * BPe + b + 1;  // psi(y, x); +-1: y, +-BPe: x
                const float* gq = qs + (l * Nx + x) * BPq + b + 2;
                const float* L = lq + (l * Nx + x) * BPe + b + 1;
                float d = l == 0 ? wr : 0.f;
                if (!ring) {
                    const float fE = f[BPe], fW = f[-BPe], fN = f[1], fS = f[-1];
                    const float fNE = f[BPe + 1], fNW = f[-BPe + 1], fSE = f[BPe - 1], fSW = f[-BPe - 1];
                    const float gE = gq[BPq], gW = gq[-BPq], gN = gq[1], gS = gq[-1];
                    const float gNE = gq[BPq + 1], gNW = gq[-BPq + 1], gSE = gq[BPq - 1], gSW = gq[-BPq - 1];
                    const float dfx = fE - fW, dfy = fN - fS, dgx = gE - gW, dgy = gN - gS;
                    const float jpp = dfx * dgy - dfy * dgx;
                    const float jpx = (fE * (gNE - gSE) - fW * (gNW - gSW)) + (fS * (gSE - gSW) - fN * (gNE - gNW));
                    const float fNd = fNE - fNW, fSd = fSE - fSW;
                    const float jxp = (gN * fNd - gS * fSd) + (gW * (fNW - fSW) - gE * (fNE - fSE));
                    const float Jb = (4.f * dfx + (fNd + fSd)) * b12;
                    float v = -(jpp + jpx + jxp) * i12 - Jb;
                    if (l == NL - 1) {
                        const float f0 = f[0];
                        v -= kappa * ((fE + fW - 2.f * f0) * idx2 + (fN + fS - 2.f * f0) * idy2);
                    }
                    const float L0 = L[0];
                    v += nu * L0;
                    v -= nu4 * ((L[BPe] + L[-BPe] - 2.f * L0) * idx2 + (L[1] + L[-1] - 2.f * L0) * idy2);
                    d += v;
                }
                const float yv = y0b[(l * Nx + x) * BPy + b];
                const float v = ring ? (fin ? yv + dt * d : 0.f) : sa * yv + sb * (gq[0] + dt * d);
                bad |= !isfinite(v);
                yn[l] = v;
            }
#pragma unroll
            for (int l = 0; l < NL; ++l) {
                // the next stage input carries a zero ring (the BC of every stage input)
                const float v = ring ? 0.f : yn[l];
                const int o = (l * Nx + x) * BPq + b + 2;
                sm[qn_off + o] = v;
                if (b < 2 && has_up) cl_st(cl_map(sm + qn_off + (l * Nx + x) * BPq + g.By + 2 + b, up), v);
                if (b >= Bc - 2 && has_down) cl_st(cl_map(sm + qn_off + (l * Nx + x) * BPq + b - Bc + 2, down), v);
                if (fin) y0b[(l * Nx + x) * BPy + b] = yn[l];
            }
#pragma unroll
            for (int m = 0; m < NL; ++m) {
                float s = 0.f;
#pragma unroll
                for (int l = 0; l < NL; ++l) s = fmaf(T.cl[m * NL + l], yn[l], s);
                op[(m * Nx + x) * BPy + b] = ring ? 0.f : s;
            }
        }
    }
}

template <int NL>
__global__ void __launch_bounds__(kClThreads, 1) k_cluster(ClusterArgs a) {
    extern __shared__ __align__(16) float sm[];
    const int C = (int)cl_size(), c = (int)cl_rank();
    const int member = blockIdx.x / C;
    const MemberDev& M = a.members[member];
    const int Ny = M.Ny, Nx = M.Nx;
    const ClGeom g = cl_geom(NL, Ny, Nx, C);
    const int tid = threadIdx.x, nt = blockDim.x;
    const int y0 = c * g.By, Bcy = max(0, min(g.By, Ny - y0));
    const int x0 = c * g.Bx, Bcx = max(0, min(g.Bx, Nx - x0));
    const float* P = a.params + (int64_t)member * QG_NPARAMS;
    float* q = a.q + M.off_state;  // [NL][Ny][Nx]
    ClConst K;
    K.Ny = Ny;
    K.Nx = Nx;
    K.barotropic = M.barotropic;
    K.idx2 = M.inv_dx2;
    K.idy2 = M.inv_dy2;
    K.i12 = M.inv_12dxdy;
    K.b12 = M.beta_12dx;
    K.nu = P[QG_P_NU];
    K.kappa = P[QG_P_KAPPA];
    K.nu4 = P[QG_P_NU4];
    K.wind_s = P[QG_P_TAU0] * M.invH0;
    for (int i = tid; i < g.total; i += nt) sm[i] = 0.f;
    __syncthreads();
    const ClTables<NL> T = cl_tables<NL>(sm, g, Ny, Nx);
    {
        float* c = sm + g.o_const;
        for (int i = tid; i < NL * NL; i += nt) {
            const int r = i / NL, m = i % NL;
            c[i] = M.Cm2l[r * kMaxLayers + m];
            c[NL * NL + i] = M.Cl2m[r * kMaxLayers + m];
        }
        for (int i = tid; i < NL; i += nt) c[2 * NL * NL + i] = M.lam[i];
        float* F = c + 2 * NL * NL + NL;
        for (int i = tid; i < Ny; i += nt) {
            F[i] = M.F[i];
            F[Ny + Nx + i] = M.ey[i];
        }
        for (int i = tid; i < Nx; i += nt) F[Ny + i] = M.ex[i];
    }
    // folded DST-I matrices: rows k < ceil(N / 2), pitch NP
    for (int i = tid; i < g.Hx * g.NPx; i += nt) {
        const int n = i % g.NPx, k = i / g.NPx;
        sm[g.o_sx + i] = n < Nx ? M.Sx[(int64_t)k * M.Px + n] : 0.f;
    }
    if (!g.share_s)
        for (int i = tid; i < g.Hy * g.NPy; i += nt) {
            const int n = i % g.NPy, k = i / g.NPy;
            sm[g.o_sy + i] = n < Ny ? M.Sy[(int64_t)k * M.Py + n] : 0.f;
        }
    // the state (own rows) and the first stage input (own rows and two-row halos, zero ring)
    for (int i = tid; i < Nx * (Bcy + 4); i += nt) {
        const int bq = i % (Bcy + 4), x = i / (Bcy + 4), y = y0 - 2 + bq;
        if (y < 0 || y >= Ny || Bcy == 0) continue;
        const bool ring = ring_cell(y, x, Ny, Nx);
#pragma unroll
        for (int l = 0; l < NL; ++l) {
            const float v = q[((int64_t)l * Ny + y) * Nx + x];
            sm[g.o_q0 + (l * Nx + x) * g.BPq + bq] = ring ? 0.f : v;
            if (bq >= 2 && bq < Bcy + 2) sm[g.o_y0 + (l * Nx + x) * g.BPy + bq - 2] = (a.apply_bc && ring) ? 0.f : v;
        }
    }
    __syncthreads();
    for (int i = tid; i < Nx * Bcy; i += nt) {
        const int b = i % Bcy, x = i / Bcy;
        float v[NL];
#pragma unroll
        for (int l = 0; l < NL; ++l) v[l] = sm[g.o_q0 + (l * Nx + x) * g.BPq + b + 2];
#pragma unroll
        for (int m = 0; m < NL; ++m) {
            float s = 0.f;
#pragma unroll
            for (int l = 0; l < NL; ++l) s = fmaf(T.cl[m * NL + l], v[l], s);
            sm[g.o_rb + (m * Nx + x) * g.BPy + b] = s;  // zero ring: v is zero there
        }
    }
    __syncthreads();
    cl_sync();  // every CTA of the cluster is running and initialised before remote stores
    bool bad = false;
    int cur = 0;
    for (int step = 0; step < a.n_steps; ++step) {
        for (int k = 0; k < a.n_stages; ++k) {
            // G1: operand rows (l, y) contract x -> (l, y, kx) at the kx owners
            dst_pass<NL, false, false>(sm, g, T, sm + g.o_rb, Nx, Bcy, g.BPy, sm + g.o_sx, g.NPx, y0, Ny, g.Bx,
                                       g.BPx, g.o_ra);
            cl_sync();
            // G2: rows (l, kx) contract y, divide -> (l, kx, ky) at the ky owners
            dst_pass<NL, true, false>(sm, g, T, sm + g.o_ra, Ny, Bcx, g.BPx, sm + g.o_sy, g.NPy, x0, Nx, g.By,
                                      g.BPy, g.o_rb);
            cl_sync();
            // G3: rows (l, ky) contract kx -> (l, ky, x) at the x owners
            dst_pass<NL, false, false>(sm, g, T, sm + g.o_rb, Nx, Bcy, g.BPy, sm + g.o_sx, g.NPx, y0, Ny, g.Bx,
                                       g.BPx, g.o_ra);
            cl_sync();
            // G4: rows (l, x) contract ky -> psi_hat (l, x, y) at the y owners and their halos
            dst_pass<NL, false, true>(sm, g, T, sm + g.o_ra, Ny, Bcx, g.BPx, sm + g.o_sy, g.NPy, x0, Nx, g.By,
                                      g.BPe, g.o_psi);
            cl_sync();
            const bool fin = k == a.n_stages - 1;
            const int qs = cur ? g.o_q1 : g.o_q0, qn = cur ? g.o_q0 : g.o_q1;
            cl_stencil<NL>(sm, g, K, T, c, y0, Bcy, qs, qn, a.sa[k], a.sb[k], a.dt, fin, bad);
            cur ^= 1;
            // no cluster barrier here: the next G1 reads only this CTA's operand rows (a CTA
            // barrier suffices), and the stencil's halo stores are read after four barriers
            __syncthreads();
        }
    }
    cl_sync();  // the last stencil's halo stores land before any CTA of the cluster exits
    for (int i = tid; i < Nx * Bcy; i += nt) {
        const int b = i % Bcy, x = i / Bcy, y = y0 + b;
#pragma unroll
        for (int l = 0; l < NL; ++l) q[((int64_t)l * Ny + y) * Nx + x] = sm[g.o_y0 + (l * Nx + x) * g.BPy + b];
    }
    if (__syncthreads_or(bad) && tid == 0 && a.flags) atomicOr(a.flags, 1);
}

using ClusterKernel = void (*)(ClusterArgs);
constexpr ClusterKernel kCluster[kMaxLayers] = {k_cluster<1>, k_cluster<2>, k_cluster<3>, k_cluster<4>,
                                                k_cluster<5>, k_cluster<6>, k_cluster<7>, k_cluster<8>};

}  // namespace

// Largest cluster size (16, 8, 4 or 2) that runs members of nl layers on an Ny x Nx grid:
// blocks of at least two rows, the shared memory of cl_geom within the device's opt-in limit,
// and at least one such cluster resident.  0 when none does.
int cluster_size_for(int nl, int Ny, int Nx, size_t* smem_bytes) {
    if (nl < 1 || nl > kMaxLayers) return 0;
    int dev = 0, optin = 0;
    if (cudaGetDevice(&dev) || cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) return 0;
    const ClusterKernel k = kCluster[nl - 1];
    for (int C = 16; C >= 2; C /= 2) {
        const ClGeom g = cl_geom(nl, Ny, Nx, C);
        const size_t bytes = (size_t)g.total * sizeof(float);
        if (g.By < 2 || bytes > (size_t)optin) continue;
        if (cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes)) continue;
        if (C > 8 && cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1)) continue;
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3((unsigned)C);
        cfg.blockDim = dim3(kClThreads);
        cfg.dynamicSmemBytes = bytes;
        cudaLaunchAttribute attr[1];
        attr[0].id = cudaLaunchAttributeClusterDimension;
        attr[0].val.clusterDim.x = (unsigned)C;
        attr[0].val.clusterDim.y = 1;
        attr[0].val.clusterDim.z = 1;
        cfg.attrs = attr;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaOccupancyMaxActiveClusters(&n, k, &cfg) != cudaSuccess) {
            cudaGetLastError();
            continue;
        }
        if (n < 1) continue;
        if (smem_bytes) *smem_bytes = bytes;
        return C;
    }
    cudaGetLastError();
    return 0;
}

// Advance every member (all with nl layers) n_steps Shu-Osher steps, one cluster of C CTAs
// per member; q in the caller's packing, in place.
cudaError_t launch_cluster(const MemberDev* members, int n_members, int nl, int C, size_t smem, float* q,
                           const float* params, int apply_bc, int n_steps, int n_stages, const float* sa,
                           const float* sb, float dt, int* flags, cudaStream_t s) {
    if (nl < 1 || nl > kMaxLayers || C < 2 || n_stages < 1 || n_stages > 4) return cudaErrorInvalidValue;
    // plans of other sizes may have set the kernel's shared-memory limit since
    cudaError_t e = cudaFuncSetAttribute(kCluster[nl - 1], cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e) return e;
    ClusterArgs a{};
    a.members = members;
    a.q = q;
    a.params = params;
    a.apply_bc = apply_bc;
    a.n_steps = n_steps;
    a.n_stages = n_stages;
    for (int k = 0; k < n_stages; ++k) {
        a.sa[k] = sa[k];
        a.sb[k] = sb[k];
    }
    a.dt = dt;
    a.flags = flags;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)(C * n_members));
    cfg.blockDim = dim3(kClThreads);
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeClusterDimension;
    attr[0].val.clusterDim.x = (unsigned)C;
    attr[0].val.clusterDim.y = 1;
    attr[0].val.clusterDim.z = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kCluster[nl - 1], a);
}

}  // namespace qg
