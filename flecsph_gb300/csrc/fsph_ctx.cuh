// fsph_ctx.cuh -- the context behind the opaque fsph_ctx handle of
// include/fsph.h, shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>

#include <string>
#include <vector>

#include "fsph_internal.cuh"

namespace fsph {
struct TimerRec {
  int phase;
  int e0, e1;
};
}  // namespace fsph

struct fsph_ctx {
  fsph_params p;
  fsph::PhysParams pp;
  int device = 0;
  int nsm = 152;
  cudaStream_t stream = nullptr;
  int64_t cap = 0;
  int n = 0;
  fsph::Particles P{}, Palt{};
  double * cs_new = nullptr;
  unsigned long long * skeys = nullptr;
  unsigned long long * skeys_tmp = nullptr;
  int * svals = nullptr;
  int * svals_tmp = nullptr;
  unsigned * hist = nullptr;
  unsigned long long * d_range = nullptr;
  fsph::Tree T{};
  fsph::Lists Ls{};
  fsph::Packed K{};
  bool mixed = false;
  fsph::GravBuffers grav{};  // allocated when enable_fmm
  bool grav_nodes_ok = false;  // grav.gn holds the multipoles of the current tree
  // multi-rank gravity: exported / imported cell records (10 doubles each),
  // grown on demand, freed with the context
  double * let_buf = nullptr;
  long long let_cap = 0;
  unsigned long long * let_count = nullptr;
  // periodic boundaries: real particles hold ids [0, nreal)
  bool periodic = false;
  long long nreal = 0;
  fsph::PeriodicScratch PS{};
  fsph::DevTime * d_time = nullptr;
  fsph::DevStatus * d_status = nullptr;
  double * d_cons = nullptr;
  int64_t iteration = 0;
  unsigned permute_skip = 0;  // fields the next permute may leave behind
  bool tree_ok = false;
  // K.ahyd holds the pressure-only acceleration of the current positions,
  // P/rho^2, v_half and alpha (set by the float-float acceleration pass,
  // cleared by every call that changes one of them)
  bool ahyd_ok = false;
  // K.fv1/fv2 hold v_half (high and low words), rho and c_s of the current
  // state (written by the float-float density pass); K.fdv holds v - v_half
  // and m (written by the float-float acceleration pass with the kick).
  // Cleared by every call that changes one of those fields.
  bool fv_ok = false;
  bool fdv_ok = false;
  // K.vel holds v and c_s of the current state (written by the permute of
  // update_iteration on the mixed path)
  bool vel_ok = false;
  bool uploaded = false;
  long long launches = 0;
  // timers
  bool timing = false;
  std::vector<cudaEvent_t> events;
  int ev_used = 0;
  std::vector<fsph::TimerRec> pending;
  double timer_ms[FSPH_TIMER_COUNT] = {0};
  long long timer_calls[FSPH_TIMER_COUNT] = {0};
  std::string last_error;
  std::vector<void *> allocs;
  cudaEvent_t marks[64] = {};
  // fsph_step_io: a copy stream, the output view of the step in progress
  // and which of its fields are already on their way to the host
  struct Io {
    cudaStream_t stream = nullptr;
    // ev[1..5]: the stages of the step; ev[0]: late input fields copied;
    // ev[6]: copies may start; ev[7]: the copy stream's work is done
    cudaEvent_t ev[8] = {};
    bool active = false;
    bool h2d_pending = false;  // late input fields on the copy stream
    fsph_soa_view out{};
    bool sent[fsph::NF + 2] = {};  // NF fields, then id, key
  } io;

  fsph::Launch L() { return fsph::Launch{stream, &launches}; }
};
