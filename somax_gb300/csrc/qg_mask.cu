// Device side of the masked-basin inversion: the capacitance correction between the two DST
// solves (host construction and the method in qg_capacitance.cu).
//
// One CTA per (member, mode, block of kCapRows rows of C^-1): it gathers psi_hat of the first
// solve at the member's boundary points B into shared memory (FP64), then each warp forms
// sigma_r = -sum_j Cinv[r][j] psi_hat[B_j] for its rows with coalesced row reads and a warp
// reduction in FP64, and adds sigma_r at B_r to the GEMM operand of the next solve (zero there
// before the first correction: B is land) and to its FP32 copy.  A repeated correction
// removes what the FP32 / split-BF16 solve leaves of psi on B after the first.  The C^-1 read dominates: 8 k^2
// bytes per mode, the kernel's HBM roofline.
#include <cuda_bf16.h>

#include "qg_device.cuh"
#include "qg_internal.cuh"

namespace qg {

namespace {

constexpr int NT = 256;

__global__ void __launch_bounds__(NT) k_capacitance(const MemberDev* __restrict__ members,
                                                    const CapItem* __restrict__ items, const float* __restrict__ psi_hat,
                                                    void* xa, int xa_fmt, float* xq, int64_t xplane) {
    extern __shared__ double v[];
    const CapItem it = items[blockIdx.x];
    const MemberDev& M = members[it.member];
    const int k = M.nb, m = it.mode;
    const int Nx = M.Nx;
    const float* ph = psi_hat + M.off_x + (int64_t)m * M.Ny * M.Px;
    for (int j = threadIdx.x; j < k; j += NT) {
        const int b = M.bidx[j];
        v[j] = (double)ph[(int64_t)(b / Nx) * M.Px + (b % Nx)];
    }
    __syncthreads();
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const double* C = M.cinv + (size_t)m * k * k;
    for (int rr = warp; rr < kCapRows; rr += NT / 32) {
        const int r = it.r0 + rr;
        if (r >= k) break;
        const double* row = C + (size_t)r * k;
        double s = 0.0;
        for (int j = lane; j < k; j += 32) s = fma(row[j], v[j], s);
        for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
        if (lane == 0) {
            // accumulate: a repeated correction adds to the sources already at B
            const int b = M.bidx[r];
            const int64_t o = M.off_x + ((int64_t)m * M.Ny + b / Nx) * M.Px + (b % Nx);
            if (xa_fmt == FMT_F32) {
                float* p = static_cast<float*>(xa);
                p[o] = (float)((double)p[o] - s);
            } else {
                __nv_bfloat16* p = static_cast<__nv_bfloat16*>(xa);
                const double cur = (double)__bfloat162float(p[o]) + (double)__bfloat162float(p[xplane + o]);
                const float sig = (float)(cur - s);
                const __nv_bfloat16 hi = __float2bfloat16_rn(sig);
                p[o] = hi;
                p[xplane + o] = __float2bfloat16_rn(sig - __bfloat162float(hi));
            }
            if (xq) xq[o] = (float)((double)xq[o] - s);
        }
    }
}

}  // namespace

cudaError_t launch_capacitance(const MemberDev* members, const CapItem* items, int n_items, const float* psi_hat,
                               void* xa, int xa_fmt, float* xq, int64_t xplane, size_t smem, cudaStream_t s) {
    if (n_items <= 0) return cudaSuccess;
    k_capacitance<<<n_items, NT, smem, s>>>(members, items, psi_hat, xa, xa_fmt, xq, xplane);
    return cudaGetLastError();
}

cudaError_t capacitance_init(size_t max_smem) {
    return cudaFuncSetAttribute(k_capacitance, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)max_smem);
}

}  // namespace qg
