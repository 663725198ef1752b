// fsph_ensemble.cu -- many independent problems on one GPU, stepped as CUDA
// graphs.
//
// The reference runs one problem per MPI job (app/drivers/hydro/
// main_driver.cc); a parameter study is many such jobs.  Here an ensemble
// holds one fsph_ctx per problem (own stream, own device arrays) and steps
// them all with one graph launch per lane and step:
//   * each member runs its initial iteration and one regular iteration
//     eagerly (this also sets every kernel attribute before any capture);
//   * then regular iterations of every member are captured one after the
//     other until every member's buffer pointers are back where they
//     started: the sort writes into the spare particle arrays (period 2)
//     and the density pass into the spare sound-speed array, which rotates
//     through three arrays with the first (period 3), so a cycle is six
//     captured iterations; the member graphs of one iteration become child
//     nodes of one root graph per lane and cycle position;
//   * a step launches the root graph of the current cycle position on every
//     lane and moves each member's host-side view (buffer pointers,
//     iteration, launch count) to where that iteration leaves it.
// Members are spread over lanes (one stream each) by particle count, largest
// first onto the least loaded lane; fsph_ensemble_tune times a few steps per
// lane count and keeps the fastest, fsph_ensemble_tune_shape does so for each
// walk-group size (8, 16, 32 particles per warp) as well.
//
// Periodic members (their copy count is read back every iteration) and
// members with timers on run eagerly, member by member.  Any host-visible
// change to a member between steps (upload, a manual pass, set_time) is
// detected and the graphs are captured again.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <cstring>
#include <numeric>
#include <string>
#include <vector>

#include "fsph_ctx.cuh"

namespace {

struct HostView {
  fsph::Particles P, Palt;
  double * cs_new;
  int n;
  bool tree_ok;
};

HostView view_of(const fsph_ctx * c) {
  return HostView{c->P, c->Palt, c->cs_new, c->n, c->tree_ok};
}

void apply_view(fsph_ctx * c, const HostView & v) {
  c->P = v.P;
  c->Palt = v.Palt;
  c->cs_new = v.cs_new;
  c->n = v.n;
  c->tree_ok = v.tree_ok;
}

bool same_particles(const fsph::Particles & a, const fsph::Particles & b) {
  for(int k = 0; k < fsph::NF; ++k)
    if(a.f[k] != b.f[k])
      return false;
  return a.id == b.id && a.key == b.key && a.n == b.n;
}

bool same_view(const HostView & a, const HostView & b) {
  return same_particles(a.P, b.P) && same_particles(a.Palt, b.Palt) &&
         a.cs_new == b.cs_new && a.n == b.n;
}

struct Member {
  fsph_ctx * c = nullptr;
  int lane = 0;
  // host view before each captured iteration of the cycle
  std::vector<HostView> at;
  std::vector<long long> launches_per_step;
  int64_t next_iteration = 0;  // iteration the next graph step starts from
};

}  // namespace

struct fsph_ensemble {
  int device = 0;
  std::vector<Member> m;
  int lanes = 1;
  bool lanes_assigned = false;
  bool eager = false;  // lanes set to 0: no graphs, every member on its own
  std::vector<cudaStream_t> lane_stream;
  std::vector<std::vector<cudaGraphExec_t>> exec;  // [cycle position][lane]
  int cycle = 0;
  std::vector<cudaEvent_t> lane_done;
  std::vector<cudaEvent_t> member_ready;
  bool graphs = false;
  int parity = 0;  // position in the cycle
  std::string last_error;
};

namespace {

fsph_status ens_cuda(fsph_ensemble * e, cudaError_t err, const char * where) {
  e->last_error = std::string(where) + ": " + cudaGetErrorString(err);
  return err == cudaErrorMemoryAllocation ? FSPH_ERR_OOM : FSPH_ERR_CUDA;
}

#define ECK(expr)                                                              \
  do {                                                                         \
    cudaError_t e_ = (expr);                                                   \
    if(e_ != cudaSuccess)                                                      \
      return ens_cuda(e, e_, #expr);                                           \
  } while(0)

void drop_graphs(fsph_ensemble * e) {
  for(auto & v : e->exec)
    for(auto & x : v)
      if(x)
        cudaGraphExecDestroy(x);
  e->exec.clear();
  e->cycle = 0;
  e->graphs = false;
}

fsph_status set_lanes(fsph_ensemble * e, int lanes) {
  e->eager = lanes == 0;
  lanes = std::max(1, std::min(lanes, (int)std::max<size_t>(1, e->m.size())));
  drop_graphs(e);
  while((int)e->lane_stream.size() < lanes) {
    cudaStream_t s;
    cudaEvent_t ev;
    ECK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    ECK(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    e->lane_stream.push_back(s);
    e->lane_done.push_back(ev);
  }
  e->lanes = lanes;
  // largest first onto the least loaded lane
  std::vector<int> order(e->m.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(),
    [&](int a, int b) { return e->m[a].c->n > e->m[b].c->n; });
  std::vector<long long> load(lanes, 0);
  for(int k : order) {
    int best = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    e->m[k].lane = best;
    load[best] += e->m[k].c->n;
  }
  e->lanes_assigned = true;
  return FSPH_OK;
}

// Relaxation iterations run eagerly: their extra passes depend on the
// iteration number, which a captured graph would freeze.
bool graph_ready(const fsph_ctx * c) {
  return c->uploaded && !c->periodic && !c->timing &&
         c->iteration > c->p.initial_iteration + 1 &&
         c->iteration >= c->p.relaxation_steps;
}

// Capture one regular iteration of every member from its current host view,
// into one root graph per lane.  The host views advance as if the iteration
// ran; the caller restores them.
fsph_status capture_parity(fsph_ensemble * e, int parity) {
  std::vector<cudaGraph_t> root(e->lanes, nullptr);
  for(int l = 0; l < e->lanes; ++l)
    ECK(cudaGraphCreate(&root[l], 0));
  fsph_status st = FSPH_OK;
  for(auto & mb : e->m) {
    fsph_ctx * c = mb.c;
    if((int)mb.at.size() <= parity) {
      mb.at.resize(parity + 1);
      mb.launches_per_step.resize(parity + 1);
    }
    mb.at[parity] = view_of(c);
    const long long l0 = c->launches;
    cudaGraph_t g = nullptr;
    cudaError_t err = cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal);
    if(err != cudaSuccess) {
      st = ens_cuda(e, err, "cudaStreamBeginCapture");
      break;
    }
    fsph_status s = fsph_step(c);
    err = cudaStreamEndCapture(c->stream, &g);
    if(s != FSPH_OK || err != cudaSuccess || !g) {
      if(g)
        cudaGraphDestroy(g);
      e->last_error = s ? std::string("capture: ") + fsph_status_string(s)
                        : std::string("capture: ") + cudaGetErrorString(err);
      cudaGetLastError();
      st = s ? s : FSPH_ERR_CUDA;
      break;
    }
    mb.launches_per_step[parity] = c->launches - l0;
    cudaGraphNode_t node;
    err = cudaGraphAddChildGraphNode(&node, root[mb.lane], nullptr, 0, g);
    cudaGraphDestroy(g);
    if(err != cudaSuccess) {
      st = ens_cuda(e, err, "cudaGraphAddChildGraphNode");
      break;
    }
  }
  if(st == FSPH_OK) {
    if((int)e->exec.size() <= parity)
      e->exec.resize(parity + 1);
    e->exec[parity].assign(e->lanes, nullptr);
    for(int l = 0; l < e->lanes && st == FSPH_OK; ++l) {
      cudaError_t err = cudaGraphInstantiate(&e->exec[parity][l], root[l], 0);
      if(err != cudaSuccess)
        st = ens_cuda(e, err, "cudaGraphInstantiate");
    }
  }
  for(auto & r : root)
    if(r)
      cudaGraphDestroy(r);
  return st;
}

fsph_status build_graphs(fsph_ensemble * e) {
  drop_graphs(e);
  std::vector<int64_t> it(e->m.size());
  std::vector<long long> la(e->m.size());
  std::vector<HostView> before(e->m.size());
  for(size_t k = 0; k < e->m.size(); ++k) {
    it[k] = e->m[k].c->iteration;
    la[k] = e->m[k].c->launches;
    before[k] = view_of(e->m[k].c);
  }
  const int max_cycle = 12;
  fsph_status st = FSPH_OK;
  bool cyclic = false;
  int len = 0;
  while(st == FSPH_OK && !cyclic && len < max_cycle) {
    st = capture_parity(e, len++);
    cyclic = true;
    for(size_t k = 0; k < e->m.size() && cyclic; ++k)
      cyclic = same_view(view_of(e->m[k].c), before[k]);
  }
  // nothing ran: put every member back where it was
  for(size_t k = 0; k < e->m.size(); ++k) {
    Member & mb = e->m[k];
    apply_view(mb.c, before[k]);
    mb.c->iteration = it[k];
    mb.c->launches = la[k];
    mb.next_iteration = it[k];
  }
  if(st != FSPH_OK) {
    drop_graphs(e);
    return st;
  }
  if(!cyclic) {
    drop_graphs(e);
    e->last_error = "a member's buffers do not return within 12 iterations";
    return FSPH_ERR_STATE;
  }
  e->graphs = true;
  e->cycle = len;
  e->parity = 0;
  return FSPH_OK;
}

// members' pending work (uploads, eager steps) before the lanes' graphs,
// and the graphs before anything later queued on a member's stream
fsph_status lanes_wait_members(fsph_ensemble * e) {
  for(size_t k = 0; k < e->m.size(); ++k) {
    ECK(cudaEventRecord(e->member_ready[k], e->m[k].c->stream));
    ECK(cudaStreamWaitEvent(e->lane_stream[e->m[k].lane], e->member_ready[k], 0));
  }
  return FSPH_OK;
}

fsph_status members_wait_lanes(fsph_ensemble * e) {
  for(int l = 0; l < e->lanes; ++l)
    ECK(cudaEventRecord(e->lane_done[l], e->lane_stream[l]));
  for(auto & mb : e->m)
    ECK(cudaStreamWaitEvent(mb.c->stream, e->lane_done[mb.lane], 0));
  return FSPH_OK;
}

bool views_match(fsph_ensemble * e) {
  for(auto & mb : e->m)
    if(!same_view(view_of(mb.c), mb.at[e->parity]) ||
       mb.c->iteration != mb.next_iteration || !graph_ready(mb.c))
      return false;
  return true;
}

}  // namespace

extern "C" {

fsph_ensemble * fsph_ensemble_create(int32_t device, fsph_status * status) {
  fsph_status dummy;
  if(!status)
    status = &dummy;
  int ndev = 0;
  if(cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    *status = FSPH_ERR_NO_DEVICE;
    return nullptr;
  }
  if(device < 0 || device >= ndev) {
    *status = FSPH_ERR_ARG;
    return nullptr;
  }
  auto * e = new fsph_ensemble();
  e->device = device;
  *status = FSPH_OK;
  return e;
}

fsph_ctx * fsph_ensemble_add(fsph_ensemble * e, const fsph_params * p,
  int64_t capacity, fsph_status * status) {
  fsph_status dummy;
  if(!status)
    status = &dummy;
  if(!e) {
    *status = FSPH_ERR_ARG;
    return nullptr;
  }
  fsph_ctx * c = fsph_create(p, e->device, capacity, status);
  if(!c)
    return nullptr;
  cudaEvent_t ev;
  if(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess) {
    fsph_destroy(c);
    *status = FSPH_ERR_CUDA;
    return nullptr;
  }
  drop_graphs(e);
  e->lanes_assigned = false;
  Member mb;
  mb.c = c;
  e->m.push_back(mb);
  e->member_ready.push_back(ev);
  return c;
}

int32_t fsph_ensemble_size(const fsph_ensemble * e) { return e ? (int32_t)e->m.size() : 0; }

fsph_ctx * fsph_ensemble_member(fsph_ensemble * e, int32_t k) {
  if(!e || k < 0 || k >= (int32_t)e->m.size())
    return nullptr;
  return e->m[k].c;
}

const char * fsph_ensemble_last_error(const fsph_ensemble * e) {
  return e ? e->last_error.c_str() : "null ensemble";
}

fsph_status fsph_ensemble_step(fsph_ensemble * e, int32_t nsteps) {
  if(!e || nsteps < 0)
    return FSPH_ERR_ARG;
  if(e->m.empty())
    return FSPH_OK;
  ECK(cudaSetDevice(e->device));
  if(!e->lanes_assigned) {
    fsph_status s = set_lanes(e, e->lanes);
    if(s)
      return s;
  }
  bool need_wait = true;       // members' own streams have queued work
  bool graph_pending = false;  // lanes hold work the members must wait for
  for(int32_t step = 0; step < nsteps; ++step) {
    bool all_ready = !e->eager;
    for(auto & mb : e->m)
      all_ready &= graph_ready(mb.c);
    if(!all_ready) {
      // eager: members that are not ready step on their own streams; the
      // others wait for the ensemble to come level
      drop_graphs(e);
      if(graph_pending) {
        fsph_status s = members_wait_lanes(e);
        if(s)
          return s;
        graph_pending = false;
      }
      need_wait = true;
      for(auto & mb : e->m) {
        fsph_status s = fsph_step(mb.c);
        if(s) {
          e->last_error = "member step: " + std::string(fsph_status_string(s)) +
                          " " + mb.c->last_error;
          return s;
        }
      }
      continue;
    }
    if(e->graphs && !views_match(e))
      drop_graphs(e);
    if(!e->graphs) {
      fsph_status s = build_graphs(e);
      if(s)
        return s;
    }
    if(need_wait) {
      fsph_status s = lanes_wait_members(e);
      if(s)
        return s;
      need_wait = false;
    }
    const int par = e->parity;
    for(int l = 0; l < e->lanes; ++l)
      ECK(cudaGraphLaunch(e->exec[par][l], e->lane_stream[l]));
    for(auto & mb : e->m) {
      apply_view(mb.c, mb.at[(par + 1) % e->cycle]);
      mb.c->iteration += 1;
      mb.c->launches += mb.launches_per_step[par];
      mb.next_iteration = mb.c->iteration;
    }
    e->parity = (par + 1) % e->cycle;
    graph_pending = true;
  }
  if(graph_pending)
    return members_wait_lanes(e);
  return FSPH_OK;
}

fsph_status fsph_ensemble_sync(fsph_ensemble * e, int32_t * failed) {
  if(!e)
    return FSPH_ERR_ARG;
  if(failed)
    *failed = -1;
  ECK(cudaSetDevice(e->device));
  for(auto s : e->lane_stream)
    ECK(cudaStreamSynchronize(s));
  for(size_t k = 0; k < e->m.size(); ++k) {
    fsph_status s = fsph_sync(e->m[k].c);
    if(s) {
      if(failed)
        *failed = (int32_t)k;
      e->last_error = "member " + std::to_string(k) + ": " + e->m[k].c->last_error;
      return s;
    }
  }
  return FSPH_OK;
}

fsph_status fsph_ensemble_set_lanes(fsph_ensemble * e, int32_t lanes) {
  if(!e || lanes < 0)
    return FSPH_ERR_ARG;
  ECK(cudaSetDevice(e->device));
  return set_lanes(e, lanes);
}

fsph_status fsph_ensemble_tune(fsph_ensemble * e, int32_t steps_per_trial,
  int32_t * lanes_chosen, double * ms_per_step) {
  if(!e || steps_per_trial < 1)
    return FSPH_ERR_ARG;
  ECK(cudaSetDevice(e->device));
  const int cands[] = {1, 2, 4, 8, 16};
  double best = 1e300;
  int best_l = e->lanes;
  for(int l : cands) {
    if(l > 1 && l > (int)e->m.size())
      break;
    fsph_status s = set_lanes(e, l);
    if(s)
      return s;
    // one step builds the graphs; then time the trial
    s = fsph_ensemble_step(e, 1);
    if(!s)
      s = fsph_ensemble_sync(e, nullptr);
    if(s)
      return s;
    auto t0 = std::chrono::steady_clock::now();
    s = fsph_ensemble_step(e, steps_per_trial);
    if(!s)
      s = fsph_ensemble_sync(e, nullptr);
    if(s)
      return s;
    double ms = std::chrono::duration<double, std::milli>(
                  std::chrono::steady_clock::now() - t0).count() / steps_per_trial;
    if(ms < best) {
      best = ms;
      best_l = l;
    }
  }
  fsph_status s = set_lanes(e, best_l);
  if(s)
    return s;
  if(lanes_chosen)
    *lanes_chosen = best_l;
  if(ms_per_step)
    *ms_per_step = best;
  return FSPH_OK;
}

fsph_status fsph_ensemble_set_group_size(fsph_ensemble * e, int32_t group_size) {
  if(!e || group_size < 0 || group_size > 32)
    return FSPH_ERR_ARG;
  ECK(cudaSetDevice(e->device));
  for(auto s : e->lane_stream)
    ECK(cudaStreamSynchronize(s));
  for(auto & mb : e->m) {
    ECK(cudaStreamSynchronize(mb.c->stream));
    mb.c->p.group_size = group_size;
  }
  // the captured iterations hold the old group size
  drop_graphs(e);
  return FSPH_OK;
}

fsph_status fsph_ensemble_tune_shape(fsph_ensemble * e, int32_t steps_per_trial,
  int32_t * lanes_chosen, int32_t * group_size_chosen, double * ms_per_step) {
  if(!e || steps_per_trial < 1)
    return FSPH_ERR_ARG;
  const int sizes[] = {8, 16, 32};
  double best = 1e300;
  int best_l = e->lanes, best_g = 32;
  for(int g : sizes) {
    fsph_status s = fsph_ensemble_set_group_size(e, g);
    if(s)
      return s;
    int32_t l = 0;
    double ms = 0;
    s = fsph_ensemble_tune(e, steps_per_trial, &l, &ms);
    if(s)
      return s;
    if(ms < best) {
      best = ms;
      best_l = l;
      best_g = g;
    }
  }
  fsph_status s = fsph_ensemble_set_group_size(e, best_g);
  if(!s)
    s = set_lanes(e, best_l);
  if(s)
    return s;
  if(lanes_chosen)
    *lanes_chosen = best_l;
  if(group_size_chosen)
    *group_size_chosen = best_g;
  if(ms_per_step)
    *ms_per_step = best;
  return FSPH_OK;
}

void fsph_ensemble_destroy(fsph_ensemble * e) {
  if(!e)
    return;
  cudaSetDevice(e->device);
  for(auto s : e->lane_stream)
    cudaStreamSynchronize(s);
  drop_graphs(e);
  for(auto & mb : e->m)
    fsph_destroy(mb.c);
  for(auto ev : e->member_ready)
    cudaEventDestroy(ev);
  for(auto ev : e->lane_done)
    cudaEventDestroy(ev);
  for(auto s : e->lane_stream)
    cudaStreamDestroy(s);
  delete e;
}

}  // extern "C"
