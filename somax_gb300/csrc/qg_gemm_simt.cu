// Plain FP32 DST-I GEMMs on the CUDA cores: the baseline ("plain FP32 single-member path")
// against which the tensor-core inversion is measured, and the fallback-free reference for
// the tcgen05 kernels' numerics.  C = A * S with S the symmetric orthonormal DST-I matrix.
#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {

namespace {

constexpr int BM = kSimtBM, BN = kSimtBN, BK = 16;
constexpr int NT = 256;

struct PassGeom {
    int Mb, K, Nn, lda, ldb, ldo;
    const float* A;
    const float* B;
    float* C;
};

__device__ __forceinline__ PassGeom pass_geom(const MemberDev& M, int pass, const void* A, void* C) {
    PassGeom g;
    const bool xin = pass_xin(pass);  // A in x-row planes, C (transposed) in y-row planes
    const bool xout = !xin;
    g.Mb = xin ? M.Ny : M.Nx;
    g.K = xin ? M.Nx : M.Ny;
    g.Nn = g.K;
    g.lda = xin ? M.Px : M.Py;
    g.ldb = g.lda;
    g.ldo = xout ? M.Px : M.Py;
    g.A = static_cast<const float*>(A) + (xin ? M.off_x : M.off_y);
    g.B = xin ? M.Sx : M.Sy;
    g.C = static_cast<float*>(C) + (xout ? M.off_x : M.off_y);
    return g;
}

template <int PASS>
__global__ void __launch_bounds__(NT) k_gemm_simt(GemmArgs ga) {
    __shared__ float As[BK][BM + 4];
    __shared__ float Bs[BK][BN + 4];
    const GemmTile t = ga.tiles[blockIdx.x];
    const MemberDev& M = ga.members[t.member];
    const PassGeom g = pass_geom(M, PASS, ga.A, ga.C);
    pdl_wait();
    pdl_launch_dependents();
    const int nl = M.nl;
    const int Mtot = nl * g.Mb;
    const int m0 = t.mt * BM, n0 = t.nt * BN;
    const int tid = threadIdx.x;
    // Interleaved ownership: rows mr + 16 i, columns nc + 16 j; the row index runs along the
    // warp so that the transposed (column-major) stores coalesce.
    const int mr = tid & 15;
    const int nc = tid >> 4;

    float acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) acc[i][j] = 0.f;

    for (int k0 = 0; k0 < g.K; k0 += BK) {
        {  // A tile: 64 rows x 16 k, 4 per thread
            const int row = tid >> 2, kq = (tid & 3) * 4;
            const int m = m0 + row;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int k = k0 + kq + c;
                As[kq + c][row] = (m < Mtot && k < g.K) ? g.A[(int64_t)m * g.lda + k] : 0.f;
            }
        }
        {  // B tile: 16 k x 64 n
            const int k = tid >> 4, nq = (tid & 15) * 4;
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int n = n0 + nq + c;
                Bs[k][nq + c] = (k0 + k < g.K && n < g.Nn) ? g.B[(int64_t)(k0 + k) * g.ldb + n] : 0.f;
            }
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < BK; ++kk) {
            float av[4], bv[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) av[i] = As[kk][mr + 16 * i];
#pragma unroll
            for (int j = 0; j < 4; ++j) bv[j] = Bs[kk][nc + 16 * j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(av[i], bv[j], acc[i][j]);
        }
        __syncthreads();
    }

#pragma unroll
    for (int i = 0; i < 4; ++i) {
        const int m = m0 + mr + 16 * i;
        if (m >= Mtot) continue;
        const int l = m / g.Mb, r = m - l * g.Mb;
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int n = n0 + nc + 16 * j;
            if (n >= g.Nn) continue;
            float v = acc[i][j];
            const int64_t o = ((int64_t)l * g.Nn + n) * g.ldo + r;
            if (PASS == G2_FWD_Y) v = v / (M.ex[r] + M.ey[n] - M.lam[l]);
            if (PASS == G4_INV_Y && ga.accumulate) v += g.C[o];
            g.C[o] = v;
        }
    }
}

}  // namespace

cudaError_t launch_gemm_simt(const GemmArgs& g, int ntiles, cudaStream_t s, bool pdl) {
    switch (g.pass) {
        case G1_FWD_X: return launch_k(k_gemm_simt<G1_FWD_X>, ntiles, NT, 0, s, pdl, g);
        case G2_FWD_Y: return launch_k(k_gemm_simt<G2_FWD_Y>, ntiles, NT, 0, s, pdl, g);
        case G3_INV_X: return launch_k(k_gemm_simt<G3_INV_X>, ntiles, NT, 0, s, pdl, g);
        case G4_INV_Y: return launch_k(k_gemm_simt<G4_INV_Y>, ntiles, NT, 0, s, pdl, g);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace qg
