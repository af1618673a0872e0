// FP32 form of the DGSEM 2-D step: placeholder until the perturbation-form kernels land.
#include "dg2d_fp32.cuh"

namespace selfgpu {
namespace dg32 {

struct State {};
State* make_state() { return new State(); }
void destroy(State* s) { delete s; }
int create(self_dg2d*, State*, const self_dg2d_desc*, const std::vector<double>&, const std::vector<double>&,
           const std::vector<double>&) {
  return set_error(nullptr, SELF_ERR_UNSUPPORTED, "FP32 form not built");
}
int set_state(self_dg2d*, State*, const double*) { return SELF_ERR_UNSUPPORTED; }
int get_state(self_dg2d*, State*, double*) { return SELF_ERR_UNSUPPORTED; }
int state_device(self_dg2d*, State*, void**, size_t*) { return SELF_ERR_UNSUPPORTED; }
int tendency(self_dg2d*, State*, double, double*) { return SELF_ERR_UNSUPPORTED; }
int rk3(self_dg2d*, State*, double, int) { return SELF_ERR_UNSUPPORTED; }
int time_kernels(self_dg2d*, State*, int, size_t, double*) { return SELF_ERR_UNSUPPORTED; }

}  // namespace dg32
}  // namespace selfgpu
