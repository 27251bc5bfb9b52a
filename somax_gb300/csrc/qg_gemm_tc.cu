// Host side of the tensor-core DST-I GEMMs: device check and the TMA descriptors of each
// (member, pass).  The kernels are in qg_persistent.cu (one pass per launch, or every pass of
// every step in one persistent launch), built from the tcgen05 blocks of qg_tc.cuh:
//
//   TF32   : kind::tf32, A and S read as float32 (the tensor core uses their top 19 bits)
//   BF16x3 : kind::f16 with bf16 operands split x = hi + lo; D += Ahi Shi + Ahi Slo + Alo Shi
#include <cstring>

#include "qg_tc.cuh"

namespace qg {

namespace {

// 2-D tensor map over `rows` rows of `cols` valid elements with a row pitch of `pitch`
// elements; columns >= cols and rows >= rows read as zero.  128-byte rows, 128-byte swizzle.
cudaError_t encode(CUtensorMap* m, const void* base, int cols, int rows, int pitch, int prec, int box_rows) {
    const bool bf = prec == QG_DST_BF16X3;
    const int es = bf ? 2 : 4;
    const uint64_t dims[2] = {(uint64_t)cols, (uint64_t)rows};
    const uint64_t strides[1] = {(uint64_t)pitch * es};
    const uint32_t box[2] = {(uint32_t)(128 / es), (uint32_t)box_rows};
    return tmap_encode(m, bf ? 1 : 0, 2, base, dims, strides, box, 1);
}

}  // namespace

cudaError_t gemm_tc_init() {
    int dev = 0, major = 0, minor = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (!e) e = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
    if (!e) e = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
    if (e) return e;
    if (major != 10 || minor != 3) return cudaErrorNotSupported;  // built for sm_103a only
    return e;
}

int gemm_tc_tile_n(int) { return TC_BN; }

// Tensor maps of one member for one pass: A from the pass's input plane(s), S of the
// contracted axis.  `a_plane` is the plane base (all members), `a_plane_elems` its size.
cudaError_t gemm_tc_encode(const MemberDev& M, int pass, const void* a_plane, int64_t a_plane_elems, int prec,
                           void* out) {
    TcMaps tm;
    std::memset(&tm, 0, sizeof(tm));
    const bool xin = pass_xin(pass);
    const int Mb = xin ? M.Ny : M.Nx, K = xin ? M.Nx : M.Ny, pitch = xin ? M.Px : M.Py;
    const int64_t off = xin ? M.off_x : M.off_y;
    const int es = prec == QG_DST_BF16X3 ? 2 : 4;
    const char* A = static_cast<const char*>(a_plane) + off * es;
    cudaError_t e = encode(&tm.a[0], A, K, M.nl * Mb, pitch, prec, TC_BM);
    if (!e && prec == QG_DST_BF16X3) e = encode(&tm.a[1], A + a_plane_elems * es, K, M.nl * Mb, pitch, prec, TC_BM);
    // S of the contracted axis: K x K, pitch = the same axis' padded length
    const void* S = prec == QG_DST_BF16X3 ? (const void*)(xin ? M.Sx_bf : M.Sy_bf) : (const void*)(xin ? M.Sx : M.Sy);
    if (!e) e = encode(&tm.b[0], S, K, K, pitch, prec, TC_BN);
    if (!e && prec == QG_DST_BF16X3)
        e = encode(&tm.b[1], static_cast<const char*>(S) + (int64_t)K * pitch * es, K, K, pitch, prec, TC_BN);
    if (!e) std::memcpy(out, &tm, sizeof(tm));
    return e;
}

}  // namespace qg
