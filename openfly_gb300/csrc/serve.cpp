// serve.cpp -- continuous batching of saddle searches (the served path).
//
// The reference runs Master::find_mechs (src/saddle/find.cpp:211-372) batch by batch: each local
// environment's searches start together and the next batch waits for the slowest. Here searches are
// requests: a host worker thread repeatedly replays one CUDA graph ("tick") that uploads the list of
// active slots, advances every active search by `steps_per_tick` translation steps with the resumable
// search kernel, and reads the slots' state back. While a tick runs, a copy stream admits queued
// requests into fresh device blocks (stream-ordered allocations, bounded by the HBM budget) and
// copies finished searches out. A request that arrives while others are on the GPU joins at the next
// tick, so its work overlaps theirs; finished slots are refilled without draining the batch. A
// search's result does not depend on what else is in flight: its state is its own and the kernel
// saves it exactly between ticks.

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "search.hpp"

namespace flygpu {
  void search_gather(BatchView const& v, std::int64_t const* d_act3_off, double* out_x, double* out_ax, cudaStream_t s);
}

using namespace flygpu;

namespace {

  using Clock = std::chrono::steady_clock;

  double ms_since(Clock::time_point a, Clock::time_point b) {
    return std::chrono::duration<double, std::milli>(b - a).count();
  }

  struct Request {
    std::uint64_t id = 0;
    SearchDev S{};
    SearchLayout layout{};
    std::vector<char> image;
    std::vector<int> mob;
    std::vector<double> pos, axis;  // inputs, all atoms
    int mode = 0;
    Clock::time_point t_submit, t_admit;
  };

  struct Slot {
    bool busy = false;
    std::unique_ptr<Request> req;
    char* block = nullptr;
  };

  struct Finished {
    flygpu_served info{};
    std::vector<double> pos, axis;
  };

}  // namespace

struct flygpu_server {
  flygpu_eam* eam = nullptr;
  SearchOpts o{};
  bool mixed = false;
  int max_active = 0, steps_per_tick = 8;
  std::int64_t budget = 0, used = 0;
  flygpu_tuning tuning{4, 256, 2, 0};
  cudaStream_t compute = nullptr, copy = nullptr;
  cudaEvent_t admitted = nullptr;
  DevBuf<SearchDev> S;
  DevBuf<int> order, n_items, work;
  PinnedBuf<SearchDev> h_S;
  PinnedBuf<int> h_order;
  std::vector<Slot> slots;
  std::deque<std::unique_ptr<Request>> pending;
  std::deque<Finished> done;
  std::map<std::uint64_t, Finished> kept;  // finished results whose positions are still wanted
  std::uint64_t next_id = 1;
  std::int64_t ticks = 0, completed = 0;
  cudaGraphExec_t graph = nullptr;
  std::mutex mu;
  std::condition_variable cv_work, cv_done;
  std::thread worker;
  bool stop = false;
  int error = FLYGPU_OK;
  std::string error_msg;

  ~flygpu_server();
  void loop();
  void tick_graph();
  void tick_body();  // the tick's work, recorded by tick_graph
  void admit(std::unique_lock<std::mutex>& lk);
  void retire();
};

namespace {

  template <typename F>
  int guard(F&& f) {
    try {
      f();
      return FLYGPU_OK;
    } catch (Error const& e) {
      set_error(e.msg);
      return e.status;
    } catch (std::bad_alloc const&) {
      set_error("host allocation failed");
      return FLYGPU_OOM;
    } catch (std::exception const& e) {
      set_error(e.what());
      return FLYGPU_INVALID_ARG;
    }
  }

}  // namespace

// One tick as a graph: upload the active list, reset the work counter, run the searches for
// steps_per_tick steps, read every slot's state back. Inactive slots are marked done on the device.
// A failure inside the capture ends it (and drops the partial graph) before the error propagates, so
// the calling thread is never left inside an open capture.
void flygpu_server::tick_graph() {
  FLY_CUDA(cudaStreamBeginCapture(compute, cudaStreamCaptureModeThreadLocal));
  try {
    tick_body();
  } catch (...) {
    cudaGraph_t dead = nullptr;
    cudaStreamEndCapture(compute, &dead);
    if (dead) cudaGraphDestroy(dead);
    cudaGetLastError();
    throw;
  }
  cudaGraph_t g = nullptr;
  FLY_CUDA(cudaStreamEndCapture(compute, &g));
  cudaError_t const e = cudaGraphInstantiate(&graph, g, 0);
  cudaGraphDestroy(g);
  FLY_CUDA(e);
}

void flygpu_server::tick_body() {
  FLY_CUDA(cudaMemcpyAsync(order.p, h_order.p, sizeof(int) * static_cast<std::size_t>(max_active + 1),
                           cudaMemcpyHostToDevice, compute));
  FLY_CUDA(cudaMemsetAsync(work.p, 0, sizeof(int), compute));
  BatchView v{};
  v.S = S.p;
  v.n_search = max_active;
  v.order = order.p + 1;
  v.n_items = max_active;  // the kernel stops at the first slot index < 0 in the list
  v.n_items_dev = order.p;
  v.work = work.p;
  v.budget = steps_per_tick;
  v.smem_bytes = SEARCH_SMEM_CAP;
  v.o = o;
  v.tb = eam->view();
  int const sms = [] {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n;
  }();
  int const blocks = std::max(1, std::min(max_active, std::max(1, tuning.blocks_per_sm) * sms));
  search_launch(v, tuning.lanes_per_atom, tuning.threads, tuning.max_registers, blocks, mixed, compute);
  FLY_CUDA(cudaMemcpyAsync(h_S.p, S.p, sizeof(SearchDev) * static_cast<std::size_t>(max_active), cudaMemcpyDeviceToHost,
                           compute));
}

flygpu_server::~flygpu_server() {
  {
    std::lock_guard<std::mutex> lk(mu);
    stop = true;
  }
  cv_work.notify_all();
  if (worker.joinable()) worker.join();
  if (compute) cudaStreamSynchronize(compute);
  if (copy) cudaStreamSynchronize(copy);
  for (auto& s : slots)
    if (s.block) cudaFree(s.block);
  if (graph) cudaGraphExecDestroy(graph);
  if (admitted) cudaEventDestroy(admitted);
  if (compute) cudaStreamDestroy(compute);
  if (copy) cudaStreamDestroy(copy);
}

// Moves queued requests into free slots while the budget allows (copy stream; caller holds lk).
void flygpu_server::admit(std::unique_lock<std::mutex>& lk) {
  (void)lk;
  bool any = false;
  for (std::size_t s = 0; s < slots.size() && !pending.empty(); ++s) {
    if (slots[s].busy) continue;
    Request& r = *pending.front();
    std::int64_t const bytes = static_cast<std::int64_t>(r.layout.total);
    if (used + bytes > budget) break;  // admission by HBM budget, in arrival order
    char* block = nullptr;
    FLY_CUDA(cudaMallocAsync(reinterpret_cast<void**>(&block), r.layout.total, copy));
    FLY_CUDA(cudaMemcpyAsync(block, r.image.data(), r.layout.total, cudaMemcpyHostToDevice, copy));
    search_bind(r.S, block, r.layout);
    FLY_CUDA(cudaMemcpyAsync(S.p + s, &r.S, sizeof(SearchDev), cudaMemcpyHostToDevice, copy));
    r.t_admit = Clock::now();
    used += bytes;
    slots[s].busy = true;
    slots[s].block = block;
    slots[s].req = std::move(pending.front());
    pending.pop_front();
    any = true;
  }
  if (any) {
    FLY_CUDA(cudaEventRecord(admitted, copy));
    FLY_CUDA(cudaStreamWaitEvent(compute, admitted, 0));
    // the host image buffers must outlive the copies
    FLY_CUDA(cudaStreamSynchronize(copy));
    for (auto& s : slots)
      if (s.busy && !s.req->image.empty()) {
        s.req->image.clear();
        s.req->image.shrink_to_fit();
      }
  }
}

// Finished slots (state read back by the last tick): copy every result out with one synchronisation,
// then free the slots.
void flygpu_server::retire() {
  struct Out {
    std::size_t slot;
    std::vector<double> x, ax;
  };
  std::vector<Out> outs;
  for (std::size_t s = 0; s < slots.size(); ++s) {
    Slot& sl = slots[s];
    if (!sl.busy || h_S.p[s].stage != STAGE_DONE) continue;
    Request& r = *sl.req;
    std::size_t const M = 3 * static_cast<std::size_t>(h_S.p[s].na);
    Out out{s, std::vector<double>(M), std::vector<double>(M)};
    double const* vec = reinterpret_cast<double const*>(sl.block + r.layout.vec);
    FLY_CUDA(cudaMemcpyAsync(out.x.data(), vec + V_X * M, M * sizeof(double), cudaMemcpyDeviceToHost, copy));
    if (r.mode == MODE_DIMER) FLY_CUDA(cudaMemcpyAsync(out.ax.data(), vec + V_AX * M, M * sizeof(double), cudaMemcpyDeviceToHost, copy));
    FLY_CUDA(cudaFreeAsync(sl.block, copy));
    outs.push_back(std::move(out));
  }
  if (outs.empty()) return;
  FLY_CUDA(cudaStreamSynchronize(copy));
  auto const now = Clock::now();
  for (Out& fin : outs) {
    Slot& sl = slots[fin.slot];
    Request& r = *sl.req;
    SearchDev const& d = h_S.p[fin.slot];
    Finished f;
    f.info.id = r.id;
    f.info.result.exit_code = d.exit_code;
    f.info.result.status = d.status;
    f.info.result.steps = d.it;
    f.info.result.grad_calls = d.grad_calls;
    f.info.result.curvature = d.curv;
    f.info.result.energy = d.energy;
    f.pos = std::move(r.pos);
    f.axis = std::move(r.axis);
    for (std::size_t k = 0; k < r.mob.size(); ++k)
      for (std::size_t c = 0; c < 3; ++c) {
        std::size_t const a = 3 * static_cast<std::size_t>(r.mob[k]) + c;
        f.pos[a] = fin.x[3 * k + c];
        if (r.mode == MODE_DIMER) f.axis[a] = fin.ax[3 * k + c];
      }
    f.info.latency_ms = ms_since(r.t_submit, now);
    f.info.queue_ms = ms_since(r.t_submit, r.t_admit);
    used -= static_cast<std::int64_t>(r.layout.total);
    sl.busy = false;
    sl.block = nullptr;
    sl.req.reset();
    ++completed;
    done.push_back(std::move(f));
  }
}

void flygpu_server::loop() {
  try {
    for (;;) {
      std::unique_lock<std::mutex> lk(mu);
      admit(lk);
      int active = 0;
      for (std::size_t s = 0; s < slots.size(); ++s)
        if (slots[s].busy) h_order.p[1 + active++] = static_cast<int>(s);
      if (active == 0) {
        if (stop) return;
        cv_work.wait(lk, [&] { return stop || !pending.empty(); });
        continue;
      }
      h_order.p[0] = active;
      lk.unlock();
      FLY_CUDA(cudaGraphLaunch(graph, compute));
      count_launch();
      FLY_CUDA(cudaStreamSynchronize(compute));
      lk.lock();
      ++ticks;
      retire();
      lk.unlock();
      cv_done.notify_all();
    }
  } catch (Error const& e) {
    std::lock_guard<std::mutex> lk(mu);
    error = e.status;
    error_msg = e.msg;
    cv_done.notify_all();
  }
}

extern "C" {

int flygpu_server_create(flygpu_eam* eam, const flygpu_dimer_options* dimer, const flygpu_lbfgs_options* lbfgs,
                         int precision, int64_t hbm_budget_bytes, int max_active, int steps_per_tick,
                         const flygpu_tuning* tuning, flygpu_server** out) {
  return guard([&] {
    if (!eam || !out) fail(FLYGPU_INVALID_ARG, "null argument");
    *out = nullptr;
    if (precision != FLYGPU_FP64 && precision != FLYGPU_MIXED) fail(FLYGPU_INVALID_ARG, "unknown precision");
    if (max_active <= 0 || steps_per_tick <= 0 || hbm_budget_bytes <= 0) fail(FLYGPU_INVALID_ARG, "bad server limits");
    flygpu_dimer_options d;
    flygpu_lbfgs_options l;
    flygpu_dimer_options_default(&d);
    flygpu_lbfgs_options_default(&l);
    if (dimer) d = *dimer;
    if (lbfgs) l = *lbfgs;
    auto srv = std::make_unique<flygpu_server>();
    srv->eam = eam;
    srv->mixed = precision == FLYGPU_MIXED;
    srv->o = make_opts(d, l, eam->r_cut);
    srv->max_active = max_active;
    srv->steps_per_tick = steps_per_tick;
    srv->budget = hbm_budget_bytes;
    if (tuning) srv->tuning = *tuning;
    {  // the launch shape must fit one SM with the server's staging budget (checked before any capture)
      flygpu_tuning const& t = srv->tuning;
      if (t.lanes_per_atom != 1 && t.lanes_per_atom != 2 && t.lanes_per_atom != 4 && t.lanes_per_atom != 8)
        fail(FLYGPU_INVALID_ARG, "lanes_per_atom must be 1, 2, 4 or 8");
      if (t.threads % 32 != 0 || t.threads < 64 || t.threads > 1024)
        fail(FLYGPU_INVALID_ARG, "threads must be 64..1024, a multiple of 32");
      int bps = 0;
      search_occupancy(t.lanes_per_atom, t.threads, srv->mixed, t.max_registers, SEARCH_SMEM_CAP, &bps);
      if (bps < 1)
        fail(FLYGPU_INVALID_ARG, "the server's launch shape does not fit an SM (threads x registers a thread, or shared "
                                 "memory): use fewer threads or max_registers = 128");
    }
    {  // keep freed request blocks in the pool instead of returning them to the driver
      int dev = 0;
      cudaMemPool_t pool;
      FLY_CUDA(cudaGetDevice(&dev));
      FLY_CUDA(cudaDeviceGetDefaultMemPool(&pool, dev));
      std::uint64_t keep = static_cast<std::uint64_t>(hbm_budget_bytes);
      FLY_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
    }
    FLY_CUDA(cudaStreamCreateWithFlags(&srv->compute, cudaStreamNonBlocking));
    FLY_CUDA(cudaStreamCreateWithFlags(&srv->copy, cudaStreamNonBlocking));
    FLY_CUDA(cudaEventCreateWithFlags(&srv->admitted, cudaEventDisableTiming));
    srv->S.reserve(static_cast<std::size_t>(max_active));
    srv->h_S.reserve(static_cast<std::size_t>(max_active));
    srv->h_order.reserve(static_cast<std::size_t>(max_active) + 1);
    srv->order.reserve(static_cast<std::size_t>(max_active) + 1);
    srv->work.reserve(1);
    std::vector<SearchDev> idle(static_cast<std::size_t>(max_active));
    for (auto& s : idle) s.stage = STAGE_DONE;
    std::memcpy(srv->h_S.p, idle.data(), sizeof(SearchDev) * idle.size());
    FLY_CUDA(cudaMemcpy(srv->S.p, idle.data(), sizeof(SearchDev) * idle.size(), cudaMemcpyHostToDevice));
    srv->slots.resize(static_cast<std::size_t>(max_active));
    search_init_kernels();  // before the capture
    srv->tick_graph();
    srv->worker = std::thread([p = srv.get()] { p->loop(); });
    *out = srv.release();
  });
}

void flygpu_server_destroy(flygpu_server* srv) { delete srv; }

namespace {

  // A request from its descriptor (validated, host copies of its arrays); throws on a bad descriptor.
  std::unique_ptr<Request> make_request(flygpu_server* srv, flygpu_search_desc const& desc) {
    auto r = std::make_unique<Request>();
    r->t_submit = Clock::now();
    r->layout = search_prepare(srv->o, srv->eam->n_types, desc, r->S, r->mob, r->image, 0);
    r->mode = desc.mode;
    r->pos.assign(desc.pos, desc.pos + 3 * desc.n);
    if (desc.mode == FLYGPU_SEARCH_DIMER) {
      r->axis.assign(desc.axis, desc.axis + 3 * desc.n);
    } else {
      r->axis.assign(static_cast<std::size_t>(3 * desc.n), 0.0);
    }
    if (static_cast<std::int64_t>(r->layout.total) > srv->budget) fail(FLYGPU_OOM, "request larger than the HBM budget");
    return r;
  }

}  // namespace

int flygpu_server_submit(flygpu_server* srv, const flygpu_search_desc* desc, uint64_t* id) {
  return flygpu_server_submit_many(srv, desc, 1, id);
}

int flygpu_server_submit_many(flygpu_server* srv, const flygpu_search_desc* descs, int n, uint64_t* ids) {
  return guard([&] {
    if (!srv || (n > 0 && !descs) || n < 0) fail(FLYGPU_INVALID_ARG, "null argument or negative count");
    std::vector<std::unique_ptr<Request>> reqs;
    reqs.reserve(static_cast<std::size_t>(n));
    for (int k = 0; k < n; ++k) {
      try {
        reqs.push_back(make_request(srv, descs[k]));
      } catch (Error const& e) {
        fail(e.status, "request " + std::to_string(k) + ": " + e.msg);
      }
    }
    std::lock_guard<std::mutex> lk(srv->mu);
    if (srv->error != FLYGPU_OK) fail(srv->error, "server stopped: " + srv->error_msg);
    for (int k = 0; k < n; ++k) {
      auto& r = reqs[static_cast<std::size_t>(k)];
      r->id = srv->next_id++;
      if (ids) ids[k] = r->id;
      srv->pending.push_back(std::move(r));
    }
    srv->cv_work.notify_one();
  });
}

int flygpu_server_poll(flygpu_server* srv, int max, int wait_ms, flygpu_served* out, int* n_out) {
  return guard([&] {
    if (!srv || !n_out || (max > 0 && !out)) fail(FLYGPU_INVALID_ARG, "null argument");
    std::unique_lock<std::mutex> lk(srv->mu);
    if (wait_ms > 0 && srv->done.empty())
      srv->cv_done.wait_for(lk, std::chrono::milliseconds(wait_ms), [&] { return !srv->done.empty() || srv->error; });
    if (srv->error != FLYGPU_OK && srv->done.empty()) fail(srv->error, "server stopped: " + srv->error_msg);
    int k = 0;
    while (k < max && !srv->done.empty()) {
      Finished& f = srv->done.front();
      out[k++] = f.info;
      srv->kept.emplace(f.info.id, std::move(f));
      srv->done.pop_front();
    }
    *n_out = k;
  });
}

int flygpu_server_take(flygpu_server* srv, uint64_t id, double* pos_out, double* axis_out) {
  return guard([&] {
    if (!srv) fail(FLYGPU_INVALID_ARG, "null server");
    std::lock_guard<std::mutex> lk(srv->mu);
    auto it = srv->kept.find(id);
    if (it == srv->kept.end()) fail(FLYGPU_INVALID_ARG, "unknown or already taken request id");
    if (pos_out) std::copy(it->second.pos.begin(), it->second.pos.end(), pos_out);
    if (axis_out) std::copy(it->second.axis.begin(), it->second.axis.end(), axis_out);
    srv->kept.erase(it);
  });
}

int flygpu_server_get_stats(flygpu_server* srv, flygpu_server_stats* st) {
  return guard([&] {
    if (!srv || !st) fail(FLYGPU_INVALID_ARG, "null argument");
    std::lock_guard<std::mutex> lk(srv->mu);
    st->pending = static_cast<int64_t>(srv->pending.size());
    int active = 0;
    for (auto const& s : srv->slots) active += s.busy;
    st->active = active;
    st->completed = srv->completed;
    st->ticks = srv->ticks;
    st->hbm_used = srv->used;
    st->hbm_budget = srv->budget;
  });
}

}  // extern "C"
