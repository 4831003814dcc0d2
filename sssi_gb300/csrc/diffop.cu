// Stand-alone staggered first derivative of a 2D or 3D column-major array
// along one dimension: the work of diffOperator_mex
// (src/fd_cmex/diffOperator_mex.c:29-213), which the MATLAB elastic and 3D
// codes call inside their time loops.
//
//   out(m) = sum_{k=0}^{order-1} c_k (in(m + order + k) - in(m + order - 1 - k)) / d
//
// along the chosen dimension, whose length shrinks by l = 2 order - 1.  One
// thread per output element, consecutive threads on consecutive elements of
// the first dimension (coalesced whichever dimension is differentiated); the
// 2 order reads of an element mostly hit L1, neighbours sharing them.
//   strict: the reference's rounding, term by term c_k * (a - b) / d with an
//           IEEE division, summed from +0 in order of k (bit-identical);
//   fused:  w_k = c_k / d folded on the host, fused multiply-adds.
#include <algorithm>

#include "api_util.cuh"
#include "divide.cuh"

namespace sssi {
namespace {

constexpr int kMaxDiffOrder = 32;

struct DiffParams {
    double c[kMaxDiffOrder];  // strict: c_k; fused: c_k / d
    Divisor<double> d;
    int order;
    int64_t n1o, n2o;  // output sizes of the first two dimensions
    int64_t jk;        // output j x k extent (second by third dimension)
    int64_t s;         // input stride of the differentiated dimension (elements)
    int64_t in_ld1, in_ld2;  // input strides of the second and third dimensions
};

template <bool STRICT>
__global__ void diffop_kernel(const double* __restrict__ in, double* __restrict__ out, const DiffParams p) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= p.n1o) return;
    for (int64_t q = blockIdx.y; q < p.jk; q += gridDim.y) {
        const int64_t j = q % p.n2o, k = q / p.n2o;
        // element (i, j, k) of the output sits at the same (i, j, k) of the input,
        // shifted along the differentiated dimension by `order` for the first term
        const double* base = in + i + j * p.in_ld1 + k * p.in_ld2 + (int64_t)p.order * p.s;
        double acc = 0.0;
        for (int t = 0; t < p.order; ++t) {
            const double a = __ldg(base + t * p.s), b = __ldg(base - (t + 1) * p.s);
            if (STRICT)
                acc = __dadd_rn(acc, div_rn(__dmul_rn(p.c[t], __dsub_rn(a, b)), p.d));
            else
                acc = fma(p.c[t], a - b, acc);
        }
        out[i + q * p.n1o] = acc;
    }
}

}  // namespace
}  // namespace sssi

using namespace sssi;

extern "C" int sssi_diffOperator(const double* data, int ndims, const int64_t* dims, const double* coeff, int order,
                                 double dist, int dim, double* out, int mode) {
    return guarded([&] {
        SSSI_REQUIRE(ndims == 2 || ndims == 3, SSSI_ERR_ARG, "diffOperator: ndims must be 2 or 3 (got %d)", ndims);
        SSSI_REQUIRE(dims && coeff, SSSI_ERR_ARG, "diffOperator: dims and coeff must not be NULL");
        SSSI_REQUIRE(dim >= 1 && dim <= ndims, SSSI_ERR_ARG, "diffOperator: dim must be in 1..%d (got %d)", ndims,
                     dim);
        SSSI_REQUIRE(order >= 1 && order <= kMaxDiffOrder, SSSI_ERR_ARG,
                     "diffOperator: 1 to %d coefficients (got %d)", kMaxDiffOrder, order);
        SSSI_REQUIRE(mode == SSSI_MODE_FP64_STRICT || mode == SSSI_MODE_FP64, SSSI_ERR_ARG,
                     "diffOperator: mode must be SSSI_MODE_FP64_STRICT or SSSI_MODE_FP64 (got %d)", mode);
        int64_t n[3] = {dims[0], dims[1], ndims == 3 ? dims[2] : 1};
        for (int a = 0; a < 3; ++a)
            SSSI_REQUIRE(n[a] >= 0 && n[a] < (int64_t(1) << 40), SSSI_ERR_ARG, "diffOperator: bad size %lld",
                         (long long)n[a]);
        const int l = 2 * order - 1;
        SSSI_REQUIRE(n[dim - 1] >= l, SSSI_ERR_ARG,
                     "diffOperator: dimension %d has %lld samples, fewer than the %d the stencil spans", dim,
                     (long long)n[dim - 1], l);
        int64_t no[3] = {n[0], n[1], n[2]};
        no[dim - 1] -= l;
        const int64_t nin = n[0] * n[1] * n[2], nout = no[0] * no[1] * no[2];
        SSSI_REQUIRE(nout == 0 || (data && out), SSSI_ERR_ARG, "diffOperator: data and out must not be NULL");
        if (nout == 0) return;
        SSSI_REQUIRE(std::isfinite(dist) && dist != 0.0, SSSI_ERR_ARG, "diffOperator: the sample distance must be "
                     "finite and nonzero");
        ensure_device();
        cudaStream_t s = current_stream();
        const bool strict = mode == SSSI_MODE_FP64_STRICT;
        DiffParams p{};
        for (int t = 0; t < order; ++t) p.c[t] = strict ? coeff[t] : coeff[t] / dist;
        p.d = make_divisor<double>(dist);
        p.order = order;
        p.n1o = no[0];
        p.n2o = no[1];
        p.jk = no[1] * no[2];
        p.in_ld1 = n[0];
        p.in_ld2 = n[0] * n[1];
        p.s = dim == 1 ? 1 : (dim == 2 ? n[0] : n[0] * n[1]);
        api::DeviceView din(data, (size_t)nin, true, s);
        api::DeviceView dout(out, (size_t)nout, false, s);
        const int threads = 128;
        const int64_t bx = (no[0] + threads - 1) / threads;
        SSSI_REQUIRE(bx < (int64_t(1) << 31), SSSI_ERR_ARG, "diffOperator: first dimension too large");
        const dim3 grid((unsigned)bx, (unsigned)std::min<int64_t>(p.jk, 65535));
        if (strict)
            diffop_kernel<true><<<grid, threads, 0, s>>>(din.ptr, dout.ptr, p);
        else
            diffop_kernel<false><<<grid, threads, 0, s>>>(din.ptr, dout.ptr, p);
        count_launch();
        SSSI_CHECK_CUDA(cudaGetLastError());
        dout.download(out, (size_t)nout, s);
        SSSI_CHECK_CUDA(cudaStreamSynchronize(s));
    });
}
