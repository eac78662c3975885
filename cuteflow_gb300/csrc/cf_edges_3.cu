/* cf_edges_3.cu -- the edge kernel of scheme IFLUX = 3 in every launch shape (cf_edge_kernel.cuh). */
#include "cf_edge_kernel.cuh"

namespace cf {
int launch_edges_3(const StepArgs& a, stream_t s) { return launch_edges_iflux<3>(a, reinterpret_cast<cudaStream_t>(s)); }
int launch_edges_list_3(const StepArgs& a, const int32_t* list, int32_t n, stream_t s) {
  return launch_edges_list_iflux<3>(a, list, n, reinterpret_cast<cudaStream_t>(s));
}
}  // namespace cf
