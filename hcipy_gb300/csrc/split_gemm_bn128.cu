// Instantiations of the split-operand tcgen05 GEMM with 128-column tiles (every output format, Babinet source
// format and embedding side), compiled on their own so the library's translation units build in parallel.
#include "split_gemm.cuh"

namespace hx {
namespace sg {

int launch_bn128(const GemmArgs& g, dim3 grid, int out, int src, cudaStream_t st) {
    return launch_out<128>(g, grid, out, src, st);
}

int cluster_ok_bn128(int ksplit) { return cluster_ok<128>(ksplit); }

}  // namespace sg
}  // namespace hx
