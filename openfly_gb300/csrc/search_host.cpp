// search_host.cpp -- host side of batched searches: layout, launch, autotuning, results.

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <sstream>
#include <string>
#include <vector>

#include "search.hpp"

namespace flygpu {

  void search_gather(BatchView const& v, std::int64_t const* d_act3_off, double* out_x, double* out_ax,
                     cudaStream_t s);

  // Options as the device sees them (all searches of a batch share them).
  SearchOpts make_opts(flygpu_dimer_options const& d, flygpu_lbfgs_options const& l, double r_cut) {
    SearchOpts o{};
    o.mT = d.n;
    o.max_steps = d.max_steps;
    o.hist_check_freq = d.hist_check_freq;
    o.use_history = d.use_history;
    o.f2norm = d.f2norm;
    o.skin_frac = d.skin_frac;
    o.proj_tol = d.proj_tol;
    o.max_trust = d.max_trust;
    o.min_trust = d.min_trust;
    o.grow_trust = d.grow_trust;
    o.shrink_trust = d.shrink_trust;
    o.convex_max = d.convex_max;
    o.mR = d.rot_n;
    o.iter_max_rot = d.iter_max_rot;
    o.relax_in_convex = d.relax_in_convex;
    o.delta_r = d.delta_r;
    o.theta_tol = d.theta_tol;
    o.mL = l.n;
    o.iter_max_l = l.iter_max;
    o.f2norm_l = l.f2norm;
    o.skin_frac_l = l.skin_frac;
    o.proj_tol_l = l.proj_tol;
    o.max_trust_l = l.max_trust;
    o.min_trust_l = l.min_trust;
    o.grow_trust_l = l.grow_trust;
    o.shrink_trust_l = l.shrink_trust;
    o.r_cut = r_cut;
    if (o.mT < 1 || o.mT > MAX_HIST || o.mR < 1 || o.mR > MAX_HIST || o.mL < 1 || o.mL > MAX_HIST)
      fail(FLYGPU_INVALID_ARG, "L-BFGS history lengths must be 1..16 on the device");
    if (o.max_steps < 0 || o.iter_max_l < 0 || o.hist_check_freq < 1) fail(FLYGPU_INVALID_ARG, "bad iteration limits");
    return o;
  }

  // List cut-offs: Dimer::find_sp (dimer.cpp:47,53) and LBFGS::minimise (lbfgs.cpp:41-45).
  double dimer_rc_list(SearchOpts const& o) {
    double const rr = o.r_cut + o.delta_r * 2;
    return rr + std::max(std::pow(o.skin_frac, 1. / 3.) - 1, 0.0) * rr;
  }
  double lbfgs_rc_list(SearchOpts const& o) {
    return o.r_cut + std::max(std::pow(o.skin_frac_l, 1. / 3.) - 1, 0.0) * o.r_cut;
  }

}  // namespace flygpu

using namespace flygpu;

struct flygpu_batch {
  flygpu_eam* eam = nullptr;
  SearchOpts o{};
  bool mixed = false;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int n_search = 0;
  std::vector<SearchDev> h_S;
  std::vector<int> order;
  std::vector<std::int64_t> n_atoms, n_mob, atom_off, act3_off;
  std::vector<double> h_pos, h_axis;  // inputs (all atoms) for assembling outputs
  std::vector<int> h_aatom;           // mobile atom -> local atom, per search at act_off
  DevBuf<SearchDev> S;
  DevBuf<int> order_d, work;
  DevBuf<char> block, block_init;  // every search's arrays (search_layout), and their initial image
  DevBuf<double> out_x, out_ax;
  DevBuf<std::int64_t> act3_d;
  std::int64_t bytes = 0;
  std::int64_t total_atoms = 0, total_act = 0;
  std::size_t block_bytes = 0;
  int smem_bytes = 0;  // dynamic shared memory per CTA for staging searches (search_smem_need, capped)
  // Two-phase runs: the whole batch for straggler_steps translation steps with the throughput shape,
  // then the unfinished searches with the wide (low-latency) shape. straggler_steps <= 0: one phase.
  int straggler_steps = 100;
  flygpu_tuning wide{4, 512, 1, 128};
  DevBuf<int> order2, n2;
  bool tuned = false;
  flygpu_tuning tuning{};
  std::string tune_key;

  BatchView view(int const* ord, int n_items, int budget, int const* n_items_dev = nullptr, int smem = -1) {
    BatchView v{};
    v.S = S.p;
    v.n_search = n_search;
    v.order = ord;
    v.n_items = n_items;
    v.n_items_dev = n_items_dev;
    v.work = work.p;
    v.budget = budget;
    v.smem_bytes = smem < 0 ? smem_bytes : smem;
    v.o = o;
    v.tb = eam->view();
    return v;
  }

  ~flygpu_batch() {
    if (stream) cudaStreamSynchronize(stream);
    if (own_stream && stream) cudaStreamDestroy(stream);
  }
};

namespace flygpu {

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

    template <typename T>
    void upload(DevBuf<T>& d, std::vector<T> const& h, cudaStream_t s) {
      d.reserve(std::max<std::size_t>(h.size(), 1));
      if (!h.empty()) FLY_CUDA(cudaMemcpyAsync(d.p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
    }

    int sm_count() {
      int dev = 0, n = 0;
      FLY_CUDA(cudaGetDevice(&dev));
      FLY_CUDA(cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev));
      return n;
    }

    std::mutex g_tune_mu;
    std::map<std::string, flygpu_tuning> g_tune_cache;

    std::string cache_path() {
      char const* p = std::getenv("FLYGPU_TUNE_CACHE");
      return p ? std::string(p) : std::string();
    }

    void load_file_cache() {
      std::string const p = cache_path();
      if (p.empty()) return;
      std::ifstream in(p);
      std::string key;
      flygpu_tuning t{};
      while (in >> key >> t.lanes_per_atom >> t.threads >> t.blocks_per_sm >> t.max_registers) g_tune_cache[key] = t;
    }

    void save_file_cache() {
      std::string const p = cache_path();
      if (p.empty()) return;
      std::ofstream out(p, std::ios::trunc);
      for (auto const& [k, t] : g_tune_cache)
        out << k << ' ' << t.lanes_per_atom << ' ' << t.threads << ' ' << t.blocks_per_sm << ' ' << t.max_registers << '\n';
    }

  }  // namespace

  // Fills S (geometry, state) for one description and writes its initial arrays into `img` at the
  // search's block offset. Returns the search's block layout. Shared by batches and the server.
  SearchLayout search_prepare(SearchOpts const& o, int n_types, flygpu_search_desc const& d, SearchDev& S,
                              std::vector<int>& mob, std::vector<char>& img, std::size_t at) {
    if (d.n <= 0 || d.n > MAX_ATOMS) fail(FLYGPU_INVALID_ARG, "atoms per search must be 1..4096");
    if (!d.pos || !d.types || !d.frozen) fail(FLYGPU_INVALID_ARG, "search without positions, types or frozen flags");
    bool const dimer = d.mode == FLYGPU_SEARCH_DIMER;
    if (!dimer && d.mode != FLYGPU_SEARCH_MINIMISE) fail(FLYGPU_INVALID_ARG, "unknown search mode");
    if (dimer && !d.axis) fail(FLYGPU_INVALID_ARG, "dimer search without an axis");
    if (d.n_hist < 0 || (d.n_hist > 0 && !d.hist)) fail(FLYGPU_INVALID_ARG, "bad saddle history");
    int const n = static_cast<int>(d.n);
    S = SearchDev{};
    S.n = n;
    S.mode = d.mode;
    S.stage = STAGE_INIT;
    S.status = FLYGPU_OK;
    S.exit_code = FLYGPU_EXIT_UNINIT;
    S.rc_list = dimer ? dimer_rc_list(o) : lbfgs_rc_list(o);
    S.theta_tol_hist = d.theta_tol;
    S.n_hist = dimer ? d.n_hist : 0;
    for (int k = 0; k < 3; ++k) {
      if (!(d.extents[k] > S.rc_list)) fail(FLYGPU_INVALID_ARG, "box extent not above the list cut-off");
      S.L[k] = d.extents[k];
      S.per[k] = d.periodic[k] ? 1 : 0;
      if (S.per[k] && !(d.extents[k] > 2 * (S.rc_list + 1e-3)))
        fail(FLYGPU_INVALID_ARG, "periodic extent must exceed twice the list cut-off in a batched search");
      S.periodic_any |= S.per[k];
      double const C = std::exp2(std::ceil(std::log2(d.extents[k] + 4 * S.rc_list + 1)));
      S.shift[k] = C + 2 * S.rc_list;
    }
    int count_frozen = 0;
    mob.clear();
    for (int i = 0; i < n; ++i) {
      if (d.types[i] >= static_cast<std::uint32_t>(n_types) || d.types[i] > 255)
        fail(FLYGPU_INVALID_ARG, "type index out of range");
      bool const fz = d.frozen[i] != 0;
      count_frozen += fz;
      bool moving = !fz;
      if (dimer && fz) moving = d.axis[3 * i] != 0 || d.axis[3 * i + 1] != 0 || d.axis[3 * i + 2] != 0;
      if (moving) mob.push_back(i);
    }
    if (mob.empty()) fail(FLYGPU_INVALID_ARG, "search without mobile atoms");
    int const na = static_cast<int>(mob.size());
    int const M = 3 * na;
    int const mT = dimer ? o.mT : o.mL, mR = dimer ? o.mR : 0;
    S.na = na;
    S.count_frozen = count_frozen;
    SearchLayout const l = search_layout(n, na, (N_VEC + 2 * mT + 2 * mR) * M, S.n_hist * (M + 2));
    if (img.size() < at + l.total) img.resize(at + l.total, 0);
    char* base = img.data() + at;
    D4* xl = reinterpret_cast<D4*>(base + l.xl);
    std::uint8_t* ty = reinterpret_cast<std::uint8_t*>(base + l.type);
    int* aat = reinterpret_cast<int*>(base + l.aatom);
    double* v = reinterpret_cast<double*>(base + l.vec);
    double* h = reinterpret_cast<double*>(base + l.hist);
    std::uint8_t* mb = reinterpret_cast<std::uint8_t*>(base + l.mob);
    std::fill_n(mb, n, std::uint8_t{0});
    for (int a : mob) mb[a] = 1;
    for (int i = 0; i < n; ++i) {
      xl[i] = D4{d.pos[3 * i], d.pos[3 * i + 1], d.pos[3 * i + 2], 0.0};
      ty[i] = static_cast<std::uint8_t>(d.types[i]);
    }
    double const* in_min = d.in_min ? d.in_min : d.pos;
    for (int k = 0; k < na; ++k) {
      int const a = mob[static_cast<std::size_t>(k)];
      aat[k] = a;
      for (int c = 0; c < 3; ++c) {
        v[V_X * M + 3 * k + c] = d.pos[3 * a + c];
        if (dimer) v[V_AX * M + 3 * k + c] = d.axis[3 * a + c];
        v[V_INMIN * M + 3 * k + c] = in_min[3 * a + c];
        for (int hh = 0; hh < S.n_hist; ++hh)
          h[hh * M + 3 * k + c] = d.hist[static_cast<std::size_t>(hh) * 3 * static_cast<std::size_t>(n) + 3 * static_cast<std::size_t>(a) + static_cast<std::size_t>(c)];
      }
    }
    // Dimer::find_sp's history check (dimer.cpp:102-131) dots x - in_min with sp - in_min over all 3n
    // coordinates. Static atoms never move in a search, so their share of both dots and of |x - in_min|^2
    // is a constant of the search (zero when the static atoms sit at in_min, as in Master's searches).
    S.hist_static_on2 = 0;
    if (S.n_hist > 0) {
      double* hs = h + static_cast<std::size_t>(S.n_hist) * static_cast<std::size_t>(M);
      for (int hh = 0; hh < S.n_hist; ++hh) hs[2 * hh] = hs[2 * hh + 1] = 0;
      for (int i = 0; i < n; ++i) {
        if (mb[i]) continue;
        for (int c = 0; c < 3; ++c) {
          double const d1 = d.pos[3 * i + c] - in_min[3 * i + c];
          S.hist_static_on2 += d1 * d1;
          for (int hh = 0; hh < S.n_hist; ++hh) {
            double const d2 = d.hist[static_cast<std::size_t>(hh) * 3 * static_cast<std::size_t>(n) + 3 * static_cast<std::size_t>(i) + static_cast<std::size_t>(c)] - in_min[3 * i + c];
            hs[2 * hh] += d1 * d2;
            hs[2 * hh + 1] += d2 * d2;
          }
        }
      }
    }
    return l;
  }

  std::vector<std::pair<std::size_t, std::size_t>> search_written(SearchLayout const& l, SearchDev const& S) {
    std::size_t const n = static_cast<std::size_t>(S.n), na = static_cast<std::size_t>(S.na), M = 3 * na;
    std::vector<std::pair<std::size_t, std::size_t>> r;
    r.emplace_back(l.xl, sizeof(D4) * n);
    r.emplace_back(l.vec + sizeof(double) * V_X * M, sizeof(double) * M);
    if (S.mode == FLYGPU_SEARCH_DIMER) r.emplace_back(l.vec + sizeof(double) * V_AX * M, sizeof(double) * M);
    r.emplace_back(l.vec + sizeof(double) * V_INMIN * M, sizeof(double) * M);
    if (S.n_hist > 0) r.emplace_back(l.hist, sizeof(double) * static_cast<std::size_t>(S.n_hist) * (M + 2));
    r.emplace_back(l.aatom, sizeof(int) * na);
    r.emplace_back(l.type, n);
    r.emplace_back(l.mob, n);
    return r;
  }

  void batch_build(flygpu_batch* B, flygpu_search_desc const* descs, int n_search) {
    if (n_search <= 0) fail(FLYGPU_INVALID_ARG, "empty batch");
    B->n_search = n_search;
    B->h_S.resize(static_cast<std::size_t>(n_search));
    // Each search is prepared in one reused scratch image; only the regions it writes go to the device
    // (most of a search's block, its neighbour columns and work vectors, starts as zeros).
    std::vector<char> scratch, compact;
    std::vector<ImageChunk> chunks;
    std::vector<SearchLayout> lay(static_cast<std::size_t>(n_search));
    std::vector<std::size_t> at(static_cast<std::size_t>(n_search));
    std::vector<std::int64_t> h_act3;
    std::vector<int> mob;
    std::size_t off = 0;
    std::int64_t atoms = 0, act = 0;
    for (int s = 0; s < n_search; ++s) {
      flygpu_search_desc const& d = descs[s];
      SearchDev& S = B->h_S[static_cast<std::size_t>(s)];
      at[static_cast<std::size_t>(s)] = off;
      lay[static_cast<std::size_t>(s)] = search_prepare(B->o, B->eam->n_types, d, S, mob, scratch, 0);
      for (auto const& [o, b] : search_written(lay[static_cast<std::size_t>(s)], S)) {
        compact.resize((compact.size() + 15) / 16 * 16);  // 8-byte aligned sources for the scatter
        chunks.push_back({static_cast<long long>(off + o), static_cast<long long>(compact.size()), static_cast<long long>(b)});
        compact.insert(compact.end(), scratch.data() + o, scratch.data() + o + b);
      }
      off += lay[static_cast<std::size_t>(s)].total;
      int const n = S.n, na = S.na;
      B->n_atoms.push_back(n);
      B->n_mob.push_back(na);
      B->atom_off.push_back(atoms);
      B->act3_off.push_back(3 * act);
      h_act3.push_back(3 * act);
      B->h_pos.insert(B->h_pos.end(), d.pos, d.pos + 3 * n);
      if (d.mode == FLYGPU_SEARCH_DIMER) {
        B->h_axis.insert(B->h_axis.end(), d.axis, d.axis + 3 * n);
      } else {
        B->h_axis.insert(B->h_axis.end(), static_cast<std::size_t>(3 * n), 0.0);
      }
      B->h_aatom.insert(B->h_aatom.end(), mob.begin(), mob.end());
      atoms += n;
      act += na;
      bool const dimer = d.mode == FLYGPU_SEARCH_DIMER;
      int const mT = dimer ? B->o.mT : B->o.mL, mR = dimer ? B->o.mR : 0;
      std::size_t const need = search_smem_need(n, static_cast<std::size_t>(N_VEC + 2 * mT + 2 * mR) * 3 * na);
      B->smem_bytes = static_cast<int>(std::min<std::size_t>(SEARCH_SMEM_CAP, std::max<std::size_t>(B->smem_bytes, need)));
    }
    search_init_kernels();
    B->total_atoms = atoms;
    B->total_act = act;
    B->block_bytes = off;
    cudaStream_t const st = B->stream;
    B->block.reserve(off);
    B->block_init.reserve(off);
    for (int s = 0; s < n_search; ++s)
      search_bind(B->h_S[static_cast<std::size_t>(s)], B->block.p + at[static_cast<std::size_t>(s)], lay[static_cast<std::size_t>(s)]);
    B->order.resize(static_cast<std::size_t>(n_search));
    std::iota(B->order.begin(), B->order.end(), 0);
    std::stable_sort(B->order.begin(), B->order.end(),
                     [&](int a, int b) { return B->n_atoms[static_cast<std::size_t>(a)] > B->n_atoms[static_cast<std::size_t>(b)]; });
    upload(B->S, B->h_S, st);
    upload(B->order_d, B->order, st);
    upload(B->act3_d, h_act3, st);
    DevBuf<char> d_compact;
    DevBuf<ImageChunk> d_chunks;
    d_compact.reserve(std::max<std::size_t>(compact.size(), 1));
    d_chunks.reserve(std::max<std::size_t>(chunks.size(), 1));
    FLY_CUDA(cudaMemsetAsync(B->block_init.p, 0, off, st));
    FLY_CUDA(cudaMemcpyAsync(d_compact.p, compact.data(), compact.size(), cudaMemcpyHostToDevice, st));
    FLY_CUDA(cudaMemcpyAsync(d_chunks.p, chunks.data(), sizeof(ImageChunk) * chunks.size(), cudaMemcpyHostToDevice, st));
    search_image_scatter(B->block_init.p, d_compact.p, d_chunks.p, static_cast<int>(chunks.size()), st);
    FLY_CUDA(cudaMemcpyAsync(B->block.p, B->block_init.p, off, cudaMemcpyDeviceToDevice, st));
    B->out_x.reserve(static_cast<std::size_t>(3 * act));
    B->out_ax.reserve(static_cast<std::size_t>(3 * act));
    B->work.reserve(1);
    B->order2.reserve(static_cast<std::size_t>(n_search));
    B->n2.reserve(1);
    FLY_CUDA(cudaStreamSynchronize(st));
    B->bytes = static_cast<std::int64_t>(B->S.n * sizeof(SearchDev) + 2 * off + 2 * B->out_x.n * 8);
    // autotune cache key: device, key version (r2: residency is tuned), precision and the size bucket
    double mean_n = static_cast<double>(atoms) / n_search, mean_a = static_cast<double>(act) / n_search;
    cudaDeviceProp prop{};
    int dev = 0;
    FLY_CUDA(cudaGetDevice(&dev));
    FLY_CUDA(cudaGetDeviceProperties(&prop, dev));
    std::ostringstream key;
    std::string name = prop.name;
    std::replace(name.begin(), name.end(), ' ', '_');
    key << name << "/r2/" << (B->mixed ? "mixed" : "fp64") << "/n" << (1 << static_cast<int>(std::lround(std::log2(std::max(1.0, mean_n)))))
        << "/a" << (1 << static_cast<int>(std::lround(std::log2(std::max(1.0, mean_a)))));
    B->tune_key = key.str();
  }

  void batch_reset(flygpu_batch* B) {
    cudaStream_t const st = B->stream;
    FLY_CUDA(cudaMemcpyAsync(B->S.p, B->h_S.data(), B->h_S.size() * sizeof(SearchDev), cudaMemcpyHostToDevice, st));
    FLY_CUDA(cudaMemcpyAsync(B->block.p, B->block_init.p, B->block_bytes, cudaMemcpyDeviceToDevice, st));
  }

  // n_items_dev: if set, the item count is read on the device (n_items is then an upper bound).
  void batch_launch(flygpu_batch* B, flygpu_tuning const& t, int const* ord, int n_items, int budget,
                    int const* n_items_dev = nullptr) {
    if (t.threads % 32 || t.threads < 32 || t.threads > 1024) fail(FLYGPU_INVALID_ARG, "bad threads per CTA");
    int const bps = std::max(1, t.blocks_per_sm);
    int const blocks = std::max(1, std::min(n_items, bps * sm_count()));
    // staging budget: the batch's largest need, or less when that keeps more CTAs resident (a search
    // stages as much of its state as fits and reads the rest from global memory)
    int const smem = search_smem_for(t.lanes_per_atom, t.threads, B->mixed, t.max_registers, bps, B->smem_bytes);
    FLY_CUDA(cudaMemsetAsync(B->work.p, 0, sizeof(int), B->stream));
    search_launch(B->view(ord, n_items, budget, n_items_dev, smem), t.lanes_per_atom, t.threads, t.max_registers,
                  blocks, B->mixed, B->stream);
  }

  // Every search of the batch to completion: one launch, or (straggler_steps > 0) a budgeted launch of
  // the whole batch followed by one of its unfinished searches in the wide shape. A search's long tail
  // then runs at the wide shape's lower latency per step instead of holding one narrow CTA.
  void batch_run_all(flygpu_batch* B, flygpu_tuning const& t) {
    if (B->straggler_steps <= 0) {
      batch_launch(B, t, B->order_d.p, B->n_search, 0);
      return;
    }
    batch_launch(B, t, B->order_d.p, B->n_search, B->straggler_steps);
    search_unfinished(B->S.p, B->order_d.p, B->n_search, B->order2.p, B->n2.p, B->stream);
    batch_launch(B, B->wide, B->order2.p, B->n_search, 0, B->n2.p);
  }

  flygpu_tuning autotune(flygpu_batch* B) {
    {
      std::lock_guard<std::mutex> lk(g_tune_mu);
      if (g_tune_cache.empty()) load_file_cache();
      auto it = g_tune_cache.find(B->tune_key);
      if (it != g_tune_cache.end()) return it->second;
    }
    // Sample: every k-th search of the size-sorted order, at least two resident waves of the GPU at the
    // highest residency tried.
    int const sms = sm_count();
    int const want = std::min(B->n_search, 12 * sms);
    std::vector<int> sample;
    for (int i = 0; i < want; ++i) sample.push_back(B->order[static_cast<std::size_t>(static_cast<std::int64_t>(i) * B->n_search / want)]);
    DevBuf<int> ord;
    upload(ord, sample, B->stream);
    cudaEvent_t e0, e1;
    FLY_CUDA(cudaEventCreate(&e0));
    FLY_CUDA(cudaEventCreate(&e1));
    flygpu_tuning best{4, 256, 2, 0};
    float best_ms = 1e30f;
    for (int lpa : {1, 2, 4, 8}) {
      for (int threads : {128, 256}) {
        for (int regs : {0, 128}) {
          // resident CTAs per SM with the full staging budget, and with none (the register limit)
          int full = 0, most = 0;
          search_occupancy(lpa, threads, B->mixed, regs, B->smem_bytes, &full);
          search_occupancy(lpa, threads, B->mixed, regs, 0, &most);
          full = std::max(1, full);
          std::vector<int> tries{full};
          if (most > full + 1) tries.push_back((full + most) / 2);
          if (most > full) tries.push_back(most);
          for (int bps : tries) {
            flygpu_tuning t{lpa, threads, bps, regs};
            batch_reset(B);
            FLY_CUDA(cudaEventRecord(e0, B->stream));
            batch_launch(B, t, ord.p, want, B->straggler_steps);  // the throughput phase
            FLY_CUDA(cudaEventRecord(e1, B->stream));
            FLY_CUDA(cudaEventSynchronize(e1));
            float ms = 0;
            FLY_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            if (ms < best_ms) {
              best_ms = ms;
              best = t;
            }
          }
        }
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    batch_reset(B);
    FLY_CUDA(cudaStreamSynchronize(B->stream));
    std::lock_guard<std::mutex> lk(g_tune_mu);
    g_tune_cache[B->tune_key] = best;
    save_file_cache();
    return best;
  }

}  // namespace flygpu

extern "C" {

void flygpu_dimer_options_default(flygpu_dimer_options* o) {
  if (!o) return;
  *o = flygpu_dimer_options{};
  o->n = 10;              // dimer.hpp:58
  o->max_steps = 1000;    // dimer.hpp:60
  o->hist_check_freq = 5; // dimer.hpp:62
  o->f2norm = 1e-5;       // dimer.hpp:64
  o->skin_frac = 1.1;     // dimer.hpp:73
  o->proj_tol = 0;
  o->max_trust = 0.5;
  o->min_trust = 0.05;
  o->grow_trust = 1.5;
  o->shrink_trust = 0.5;
  o->convex_max = 3;
  o->use_history = 1;
  o->rot_n = 6;           // rotor.hpp:49
  o->iter_max_rot = 20;   // rotor.hpp:51
  o->delta_r = 0.001;     // rotor.hpp:53
  o->theta_tol = 1 * M_PI / 360.;  // rotor.hpp:55
  o->relax_in_convex = 1;
}

void flygpu_lbfgs_options_default(flygpu_lbfgs_options* o) {
  if (!o) return;
  *o = flygpu_lbfgs_options{};
  o->n = 10;            // lbfgs.hpp:57
  o->iter_max = 2000;   // lbfgs.hpp:59
  o->f2norm = 1e-6;     // lbfgs.hpp:61
  o->skin_frac = 1.1;   // lbfgs.hpp:70
  o->proj_tol = 0;
  o->max_trust = 0.5;
  o->min_trust = 0.01;
  o->grow_trust = 1.5;
  o->shrink_trust = 0.5;
}

int flygpu_batch_create(flygpu_eam* eam, const flygpu_dimer_options* dimer, const flygpu_lbfgs_options* lbfgs,
                        int precision, const flygpu_search_desc* descs, int n_search, void* stream,
                        flygpu_batch** out) {
  return guard([&] {
    if (!eam || !descs || !out) fail(FLYGPU_INVALID_ARG, "null argument");
    *out = nullptr;
    if (precision != FLYGPU_FP64 && precision != FLYGPU_MIXED) fail(FLYGPU_INVALID_ARG, "unknown precision");
    flygpu_dimer_options d;
    flygpu_lbfgs_options l;
    flygpu_dimer_options_default(&d);
    flygpu_lbfgs_options_default(&l);
    if (dimer) d = *dimer;
    if (lbfgs) l = *lbfgs;
    auto B = std::make_unique<flygpu_batch>();
    B->eam = eam;
    B->mixed = precision == FLYGPU_MIXED;
    B->o = make_opts(d, l, eam->r_cut);
    if (stream) {
      B->stream = static_cast<cudaStream_t>(stream);
    } else {
      FLY_CUDA(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
      B->own_stream = true;
    }
    batch_build(B.get(), descs, n_search);
    *out = B.release();
  });
}

void flygpu_batch_destroy(flygpu_batch* batch) { delete batch; }

int flygpu_batch_run(flygpu_batch* B, const flygpu_tuning* tuning) {
  return guard([&] {
    if (!B) fail(FLYGPU_INVALID_ARG, "null batch");
    flygpu_tuning t;
    if (tuning) {
      t = *tuning;
    } else {
      if (!B->tuned) {
        B->tuning = autotune(B);
        B->tuned = true;
      }
      t = B->tuning;
    }
    batch_run_all(B, t);
  });
}

int flygpu_batch_set_stragglers(flygpu_batch* B, int steps, const flygpu_tuning* wide) {
  return guard([&] {
    if (!B) fail(FLYGPU_INVALID_ARG, "null batch");
    if (wide && (wide->threads % 32 || wide->threads < 64 || wide->threads > 1024))
      fail(FLYGPU_INVALID_ARG, "bad threads per CTA");
    B->straggler_steps = steps;
    if (wide) B->wide = *wide;
    B->tuned = false;  // the throughput phase is tuned with the budget
  });
}

int flygpu_batch_autotune(flygpu_batch* B, flygpu_tuning* best) {
  return guard([&] {
    if (!B || !best) fail(FLYGPU_INVALID_ARG, "null argument");
    B->tuning = autotune(B);
    B->tuned = true;
    *best = B->tuning;
  });
}

int flygpu_batch_reset(flygpu_batch* B) {
  return guard([&] {
    if (!B) fail(FLYGPU_INVALID_ARG, "null batch");
    batch_reset(B);
  });
}

int64_t flygpu_batch_device_bytes(const flygpu_batch* B) { return B ? B->bytes : 0; }

int flygpu_batch_results(flygpu_batch* B, flygpu_search_result* results, double* pos_out, double* axis_out) {
  return guard([&] {
    if (!B) fail(FLYGPU_INVALID_ARG, "null batch");
    cudaStream_t const st = B->stream;
    std::vector<SearchDev> S(static_cast<std::size_t>(B->n_search));
    FLY_CUDA(cudaMemcpyAsync(S.data(), B->S.p, S.size() * sizeof(SearchDev), cudaMemcpyDeviceToHost, st));
    std::vector<double> ox, oa;
    if (pos_out || axis_out) {
      search_gather(B->view(B->order_d.p, B->n_search, 0), B->act3_d.p, B->out_x.p, B->out_ax.p, st);
      ox.resize(static_cast<std::size_t>(3 * B->total_act));
      oa.resize(ox.size());
      FLY_CUDA(cudaMemcpyAsync(ox.data(), B->out_x.p, ox.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
      FLY_CUDA(cudaMemcpyAsync(oa.data(), B->out_ax.p, oa.size() * sizeof(double), cudaMemcpyDeviceToHost, st));
    }
    FLY_CUDA(cudaStreamSynchronize(st));
    int first_bad = FLYGPU_OK;
    std::int64_t pos_base = 0;
    for (int s = 0; s < B->n_search; ++s) {
      SearchDev const& d = S[static_cast<std::size_t>(s)];
      if (results) {
        flygpu_search_result& r = results[s];
        r.exit_code = d.exit_code;
        r.status = d.status;
        r.steps = d.it;
        r.pad_ = 0;
        r.grad_calls = d.grad_calls;
        r.curvature = d.curv;
        r.energy = d.energy;
      }
      if (d.status != FLYGPU_OK && first_bad == FLYGPU_OK) first_bad = d.status;
      std::int64_t const n = B->n_atoms[static_cast<std::size_t>(s)];
      if (pos_out || axis_out) {
        std::int64_t const a3 = B->act3_off[static_cast<std::size_t>(s)];
        std::int64_t const na = B->n_mob[static_cast<std::size_t>(s)];
        std::int64_t const a0 = a3 / 3;
        if (pos_out) std::copy_n(&B->h_pos[static_cast<std::size_t>(3 * pos_base)], 3 * n, pos_out + 3 * pos_base);
        if (axis_out) std::copy_n(&B->h_axis[static_cast<std::size_t>(3 * pos_base)], 3 * n, axis_out + 3 * pos_base);
        for (std::int64_t k = 0; k < na; ++k) {
          int const a = B->h_aatom[static_cast<std::size_t>(a0 + k)];
          for (int c = 0; c < 3; ++c) {
            if (pos_out) pos_out[3 * (pos_base + a) + c] = ox[static_cast<std::size_t>(a3 + 3 * k + c)];
            if (axis_out && d.mode == MODE_DIMER) axis_out[3 * (pos_base + a) + c] = oa[static_cast<std::size_t>(a3 + 3 * k + c)];
          }
        }
      }
      pos_base += n;
    }
    (void)first_bad;
  });
}

}  // extern "C"
