/* cf_edges_1.cu -- the edge kernel of scheme IFLUX = 1 in every launch shape (cf_edge_kernel.cuh). */
#include "cf_edge_kernel.cuh"

namespace cf {
int launch_edges_1(const StepArgs& a, stream_t s) { return launch_edges_iflux<1>(a, reinterpret_cast<cudaStream_t>(s)); }
int launch_edges_list_1(const StepArgs& a, const int32_t* list, int32_t n, stream_t s) {
  return launch_edges_list_iflux<1>(a, list, n, reinterpret_cast<cudaStream_t>(s));
}
}  // namespace cf
