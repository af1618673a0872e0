// FP32 form of the DGSEM 2-D step (declarations; kernels in dg2d_fp32.cu).
#pragma once

#include <vector>

#include "internal.hpp"

struct self_dg2d;

namespace selfgpu {
namespace dg32 {

struct State;
State* make_state();

int create(self_dg2d* h, State* s, const self_dg2d_desc* d, const std::vector<double>& met,
           const std::vector<double>& aux, const std::vector<double>& egeo);
int set_state(self_dg2d* h, State* s, const double* q);
int get_state(self_dg2d* h, State* s, double* q);
int state_device(self_dg2d* h, State* s, void** dptr, size_t* bytes);
int tendency(self_dg2d* h, State* s, double t, double* dqdt);
int rk3(self_dg2d* h, State* s, double tn, int nsteps);
int time_kernels(self_dg2d* h, State* s, int reps, size_t flush_bytes, double* ms);
// reports a bounded-wait time-out recorded by the fused stage kernel (after synchronisation)
int sync_and_check(self_dg2d* h, State* s);
// time-out test hook of the fused stage: the next call's first bulk-copy wait of every warp runs out after `polls`
int arm_wait_timeout(self_dg2d* h, State* s, int polls);
// 1 when the fused TMA-pipelined stage is in use
int is_fused(State* s);
long long bytes(const State* s);
void destroy(State* s);

}  // namespace dg32
}  // namespace selfgpu
