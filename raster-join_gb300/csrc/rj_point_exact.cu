// rj_point_exact.cu -- point passes of the index, exact (classified grid)
// and hybrid joins.  The kernels and mappers are in rj_point_core.cuh; a
// translation unit of its own so the two halves of the point kernels compile
// in parallel.
#include "rj_point_core.cuh"

namespace rj {

void launch_index_points(const PointArgs& pa, const IndexArgs& ia, int sms, cudaStream_t st) {
    IndexMapper m{ia};
    launch_points(pa, m, sms, st);
}

void launch_exact_points(const PointArgs& pa, const ExactIndex& ix, int sms, cudaStream_t st) {
    ExactMapper m{ix};
    launch_points(pa, m, sms, st);
}

void launch_hybrid_points(const PointArgs& pa, const ExactIndex& ix, const HybridArgs& ha, int sms,
                          cudaStream_t st) {
    HybridMapper m{ix, ha};
    launch_points(pa, m, sms, st);
}

}  // namespace rj
