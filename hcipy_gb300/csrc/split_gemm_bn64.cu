// Instantiations of the split-operand tcgen05 GEMM with 64-column tiles (every output format, Babinet source
// format and embedding side), compiled on their own so the library's translation units build in parallel.
#include "split_gemm.cuh"

namespace hx {
namespace sg {

int launch_bn64(const GemmArgs& g, dim3 grid, int out, int src, cudaStream_t st) {
    return launch_out<64>(g, grid, out, src, st);
}

int cluster_ok_bn64(int ksplit) { return cluster_ok<64>(ksplit); }

}  // namespace sg
}  // namespace hx
