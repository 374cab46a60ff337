// abi.cpp -- extern "C" entry points of libflygpu (declared in include/flygpu.h).

#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <new>

#include <thread>

#include "internal.hpp"

namespace flygpu {

  namespace {
    thread_local std::string g_last_error;
    std::atomic<long long> g_launches{0};
  }

  void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
  long long launch_count() { return g_launches.load(std::memory_order_relaxed); }

  void set_error(std::string msg) { g_last_error = std::move(msg); }

  void fail(int status, std::string msg) { throw Error{status, std::move(msg)}; }

  int status_from_word(int w) {
    if (w & ERR_GHOST_OVERFLOW) return FLYGPU_GHOST_OVERFLOW;
    if (w & ERR_NLIST_OVERFLOW) return FLYGPU_NLIST_OVERFLOW;
    if (w & ERR_SPLINE_OOB) return FLYGPU_SPLINE_OOB;
    if (w & ERR_TIMEOUT) return FLYGPU_TIMEOUT;
    if (w & ERR_BAD_INDEX) return FLYGPU_INVALID_ARG;
    return FLYGPU_OK;
  }

  flygpu_eam* eam_load(char const* path);

  cudaEvent_t timer_record(flygpu_list* L) {
    if (!L->timing) return nullptr;
    if (L->ev_used == L->ev_pool.size()) {
      cudaEvent_t e;
      FLY_CUDA(cudaEventCreate(&e));
      L->ev_pool.push_back(e);
    }
    cudaEvent_t const e = L->ev_pool[L->ev_used++];
    FLY_CUDA(cudaEventRecord(e, L->stream));
    return e;
  }

  void timer_mark(flygpu_list* L, int kind, cudaEvent_t a, cudaEvent_t b) {
    if (a && b) L->marks.push_back({kind, a, b});
  }

  // Runs f, converting exceptions into a status and recording the message.
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

  // Syncs the list's stream and converts its device error word into a status.
  void check_device(flygpu_list* L) {
    int const w = list_take_error(L);
    if (w) {
      int const st = status_from_word(w);
      fail(st, st == FLYGPU_SPLINE_OOB ? "spline argument outside the tabulated region"
                                       : "device-side error word " + std::to_string(w));
    }
  }

  void need(bool ok, char const* what) {
    if (!ok) fail(FLYGPU_INVALID_ARG, what);
  }

  // EAM::hessian + mass_weight + eigenvalues of the atoms of a built list (types / frozen already set;
  // the host copies are read for the masses and the active block). hess (may be NULL) receives the
  // mass-weighted matrix. Scratch stays in the list.
  void hessian_prefactor_one(flygpu_eam* eam, flygpu_list* list, uint32_t const* types, uint8_t const* frozen,
                             double const* masses, double* eig, double* hess) {
    std::size_t const N = 3 * static_cast<std::size_t>(list->n);
    if (N == 0) return;
    DevBuf<double>& H = list->hs.H;
    H.reserve(N * N);
    eam_hessian(eam, list, frozen, H.p);
    check_device(list);
    hessian_mass_weight(eam, list, masses, types, H.p);
    if (hess) {
      FLY_CUDA(cudaMemcpyAsync(hess, H.p, sizeof(double) * N * N, cudaMemcpyDeviceToHost, list->stream));
      FLY_CUDA(cudaStreamSynchronize(list->stream));
    }
    hessian_eigenvalues(list, H.p, frozen, eig);
  }

  // A list keeps its dense Hessian buffer between calls, except one above 1 GiB (a large system's matrix
  // is not held after the call that needed it).
  void release_large_hessian(flygpu_list* list) {
    if (list->hs.H.n * sizeof(double) > (std::size_t{1} << 30)) list->hs.H.release();
  }

  // The box and cut-off of a list (neigh::List::List, neigh/list.hpp:86-90; HyperGrid, hypergrid.hpp:43-53):
  // cell grid and the offset of the binary32 packed coordinates. The list must be rebuilt afterwards.
  void list_set_box(flygpu_list* L, double const extents[3], int const periodic[3], double r_cut) {
    need(r_cut > 0, "r_cut must be positive");
    GridDesc g{};
    g.rc = r_cut;
    double shift[3];
    for (int k = 0; k < 3; ++k) {
      need(extents[k] > 0, "box extents must be positive");
      need(extents[k] > r_cut, "r_cut is too big for the box");  // hypergrid.hpp:46-48
      g.L[k] = extents[k];
      g.per[k] = periodic[k] ? 1 : 0;
      g.shape[k] = 2 + static_cast<int>(extents[k] / r_cut);
      g.cell[k] = extents[k] / std::floor(extents[k] / r_cut);
      g.inv_cell[k] = 1.0 / g.cell[k];
      double const C = std::exp2(std::ceil(std::log2(extents[k] + 4 * r_cut + 1)));
      shift[k] = C + 2 * r_cut;
    }
    need(static_cast<double>(g.shape[0]) * g.shape[1] * g.shape[2] < 2e9, "too many cells");
    L->g = g;
    for (int k = 0; k < 3; ++k) L->shift[k] = shift[k];
    L->built = false;
    L->packed_valid = false;
  }

  // The device address of host memory that kernels can store to directly (pinned or registered host
  // memory, mapped into the device's address space), else null. Results written there cross the host
  // link while the kernel runs, instead of in a copy after it.
  double* device_alias(double* host) {
    cudaPointerAttributes pa{};
    int dev = 0;
    if (cudaPointerGetAttributes(&pa, host) != cudaSuccess || cudaGetDevice(&dev) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    // host memory pinned under another device's context may not be mapped for this one: copy instead
    bool const mapped_here = pa.type == cudaMemoryTypeHost && pa.devicePointer && pa.device == dev;
    return mapped_here ? static_cast<double*>(pa.devicePointer) : nullptr;
  }

  void run_eam(flygpu_eam* E, flygpu_list* L, int precision, double* d_energy, double* d_grad) {
    need(E && L, "null handle");
    need(precision == FLYGPU_FP64 || precision == FLYGPU_MIXED, "unknown precision");
    if (precision == FLYGPU_FP64) {
      eam_fp64(E, L, d_energy, d_grad);
    } else {
      eam_mixed(E, L, d_energy, d_grad);
    }
  }

}  // namespace flygpu

using namespace flygpu;

extern "C" {

const char* flygpu_status_string(int status) {
  switch (status) {
    case FLYGPU_OK: return "ok";
    case FLYGPU_INVALID_ARG: return "invalid argument";
    case FLYGPU_SPLINE_OOB: return "spline out of bounds";
    case FLYGPU_GHOST_OVERFLOW: return "ghost capacity exceeded";
    case FLYGPU_NLIST_OVERFLOW: return "neighbour capacity exceeded";
    case FLYGPU_OOM: return "out of memory";
    case FLYGPU_TIMEOUT: return "device iteration budget exhausted";
    case FLYGPU_CUDA_ERROR: return "CUDA error";
    default: return "unknown status";
  }
}

const char* flygpu_last_error(void) { return g_last_error.c_str(); }

int64_t flygpu_launch_count(void) { return launch_count(); }

int flygpu_eam_load(const char* path, flygpu_eam** out) {
  return guard([&] {
    need(path && out, "null argument");
    *out = nullptr;
    *out = eam_load(path);
  });
}

void flygpu_eam_destroy(flygpu_eam* eam) { delete eam; }

double flygpu_eam_r_cut(const flygpu_eam* eam) { return eam ? eam->r_cut : 0.0; }

int flygpu_eam_n_types(const flygpu_eam* eam) { return eam ? eam->n_types : 0; }

int64_t flygpu_eam_table(const flygpu_eam* eam, int kind, int a, int b, double* out, int64_t cap) {
  if (!eam || kind < 0 || kind > 2 || a < 0 || a >= eam->n_types || b < 0 || b >= eam->n_types) return -1;
  SplineSet const& s = kind == 0 ? eam->F : kind == 1 ? eam->phi : eam->v;
  int const fn = kind == 0 ? a : a + eam->n_types * b;
  int64_t const count = s.n_spines;
  if (out && cap >= 4 * count)
    std::memcpy(out, &s.host[static_cast<std::size_t>(fn) * static_cast<std::size_t>(count) * 4],
                sizeof(double) * static_cast<std::size_t>(4 * count));
  return count;
}

int64_t flygpu_spline_build(const double* y, int64_t n, double dx, double* out, int64_t cap) {
  if (!y || n < 2 || !(dx > 0)) {
    set_error("spline needs at least two samples and a positive spacing");
    return -1;
  }
  int const count = spline_spines(static_cast<std::size_t>(n));
  if (out && cap >= 4 * static_cast<int64_t>(count)) {
    int const st = guard([&] { build_spline(std::vector<double>(y, y + n), dx, out, count); });
    if (st != FLYGPU_OK) return -1;
  }
  return count;
}

int flygpu_list_create(const double extents[3], const int periodic[3], double r_cut, void* stream, flygpu_list** out) {
  return guard([&] {
    need(extents && periodic && out, "null argument");
    *out = nullptr;
    auto L = std::make_unique<flygpu_list>();
    list_set_box(L.get(), extents, periodic, r_cut);
    if (stream) {
      L->stream = static_cast<cudaStream_t>(stream);
    } else {
      FLY_CUDA(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking));
      L->own_stream = true;
    }
    L->err.reserve(1);
    L->counters.reserve(8);
    L->h_small.reserve(8);
    FLY_CUDA(cudaMemsetAsync(L->err.p, 0, sizeof(int), L->stream));
    FLY_CUDA(cudaStreamSynchronize(L->stream));
    *out = L.release();
  });
}

void flygpu_list_destroy(flygpu_list* list) {
  if (!list) return;
  if (list->stream) cudaStreamSynchronize(list->stream);
  bool const own = list->own_stream;
  cudaStream_t const s = list->stream;
  delete list;
  if (own) cudaStreamDestroy(s);
}

int flygpu_list_rebuild(flygpu_list* list, const double* pos, int64_t n) {
  return guard([&] {
    need(list && (pos || n == 0), "null argument");
    need(n >= 0, "negative atom count");
    list->io.reserve(static_cast<std::size_t>(3 * n + 3));
    if (n) FLY_CUDA(cudaMemcpyAsync(list->io.p, pos, sizeof(double) * 3 * static_cast<std::size_t>(n),
                                    cudaMemcpyHostToDevice, list->stream));
    list_rebuild(list, list->io.p, n);
    check_device(list);
  });
}

int flygpu_list_rebuild_device(flygpu_list* list, const double* d_pos, int64_t n) {
  return guard([&] {
    need(list && (d_pos || n == 0), "null argument");
    list_rebuild(list, d_pos, n);
  });
}

int flygpu_list_update(flygpu_list* list, const double* delta) {
  return guard([&] {
    need(list && delta, "null argument");
    std::size_t const n3 = 3 * static_cast<std::size_t>(list->n);
    // one bulk copy: the update kernel reading a pinned delta over the host link itself (per slot, ghosts
    // included) was slower, 0.24 ms against 0.17 ms for 1,023,487 atoms
    list->io.reserve(n3 + 3);
    if (n3) FLY_CUDA(cudaMemcpyAsync(list->io.p, delta, sizeof(double) * n3, cudaMemcpyHostToDevice, list->stream));
    list_update(list, list->io.p);
  });
}

int flygpu_list_update_device(flygpu_list* list, const double* d_delta) {
  return guard([&] {
    need(list && d_delta, "null argument");
    list_update(list, d_delta);
  });
}

int64_t flygpu_list_size(const flygpu_list* list) { return list ? list->n : 0; }

int64_t flygpu_list_num_ghosts(const flygpu_list* list) { return list ? list->n_slots - list->n : 0; }

int flygpu_list_neighbours(flygpu_list* list, double r_cut, int32_t* counts, int32_t* idx, double* dr, int64_t cap,
                           int64_t* total) {
  return guard([&] {
    need(list && total, "null argument");
    *total = list_export(list, r_cut, counts, idx, dr, cap);
    check_device(list);
  });
}

int flygpu_perturb(flygpu_list* nl_pert, int64_t centre, const double* in_pos, const uint8_t* frozen, int64_t n,
                   double stddev, double r_pert, flygpu_xoshiro* prng, double* out_pos, double* out_axis,
                   double* stddev_used) {
  return guard([&] {
    need(nl_pert && in_pos && frozen && prng && out_pos && out_axis, "null argument");
    need(n == nl_pert->n, "atom count differs from the list's");
    need(centre >= 0 && centre < n, "centre out of range");
    need(!frozen[centre], "perturbation centred on a frozen atom");  // find.cpp:1206
    need(r_pert > 0 && stddev > 0, "r_pert and stddev must be positive");
    std::vector<int> idx;
    std::vector<double> dr;
    int const c = list_neighbours_of(nl_pert, r_pert, centre, idx, dr);
    check_device(nl_pert);
    std::vector<double> r(static_cast<std::size_t>(c));
    for (int k = 0; k < c; ++k) {
      double const* d = &dr[3 * static_cast<std::size_t>(k)];
      r[static_cast<std::size_t>(k)] = std::sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
    }
    double const s = perturb(idx, r, centre, in_pos, frozen, n, stddev, r_pert, *prng, out_pos, out_axis);
    if (stddev_used) *stddev_used = s;
  });
}

int flygpu_list_set_timing(flygpu_list* list, int enable) {
  return guard([&] {
    need(list, "null handle");
    FLY_CUDA(cudaStreamSynchronize(list->stream));
    list->timing = enable != 0;
    list->marks.clear();
    list->ev_used = 0;
  });
}

int flygpu_list_kernel_times(flygpu_list* list, double* ms, int64_t* counts) {
  return guard([&] {
    need(list && ms && counts, "null argument");
    FLY_CUDA(cudaStreamSynchronize(list->stream));
    for (int k = 0; k < TK_COUNT; ++k) {
      ms[k] = 0;
      counts[k] = 0;
    }
    for (auto const& m : list->marks) {
      float t = 0;
      FLY_CUDA(cudaEventElapsedTime(&t, m.a, m.b));
      ms[m.kind] += t;
      counts[m.kind] += 1;
    }
    list->marks.clear();
    list->ev_used = 0;
  });
}

int flygpu_list_sync(flygpu_list* list) {
  return guard([&] {
    need(list, "null handle");
    FLY_CUDA(cudaStreamSynchronize(list->stream));
    check_device(list);
  });
}

int flygpu_eam_energy_gradient(flygpu_eam* eam, flygpu_list* list, const uint32_t* types, const uint8_t* frozen,
                               int precision, double* energy, double* grad) {
  return guard([&] {
    need(eam && list, "null handle");
    need(list->built, "EAM call before List::rebuild()");
    list_set_atoms(list, eam->n_types, nullptr, nullptr, true, types, frozen);
    std::size_t const n3 = 3 * static_cast<std::size_t>(list->n);
    list->io.reserve(n3 + 3);
    list->energy.reserve(1);
    // a pinned gradient buffer receives the force pass's stores directly (overlapped with the pass);
    // any other buffer gets a copy after it
    double* const direct = grad && n3 ? device_alias(grad) : nullptr;
    run_eam(eam, list, precision, energy ? list->energy.p : nullptr, grad ? (direct ? direct : list->io.p) : nullptr);
    if (grad && n3 && !direct)
      FLY_CUDA(cudaMemcpyAsync(grad, list->io.p, sizeof(double) * n3, cudaMemcpyDeviceToHost, list->stream));
    if (energy) FLY_CUDA(cudaMemcpyAsync(energy, list->energy.p, sizeof(double), cudaMemcpyDeviceToHost, list->stream));
    check_device(list);
  });
}

int flygpu_eam_energy(flygpu_eam* eam, flygpu_list* list, const uint32_t* types, const uint8_t* frozen, int precision,
                      double* energy) {
  if (!energy) {
    set_error("null energy pointer");
    return FLYGPU_INVALID_ARG;
  }
  return flygpu_eam_energy_gradient(eam, list, types, frozen, precision, energy, nullptr);
}

int flygpu_eam_gradient(flygpu_eam* eam, flygpu_list* list, const uint32_t* types, const uint8_t* frozen,
                        int precision, double* grad) {
  if (!grad) {
    set_error("null gradient pointer");
    return FLYGPU_INVALID_ARG;
  }
  return flygpu_eam_energy_gradient(eam, list, types, frozen, precision, nullptr, grad);
}

int flygpu_eam_hessian(flygpu_eam* eam, flygpu_list* list, const uint32_t* types, const uint8_t* frozen, double* hess) {
  return guard([&] {
    need(eam && list && hess, "null argument");
    need(list->built, "EAM call before List::rebuild()");
    need(types && frozen, "types and frozen flags are required");
    list_set_atoms(list, eam->n_types, nullptr, nullptr, true, types, frozen);
    std::size_t const N = 3 * static_cast<std::size_t>(list->n);
    if (N == 0) return;
    DevBuf<double>& H = list->hs.H;
    H.reserve(N * N);
    eam_hessian(eam, list, frozen, H.p);
    check_device(list);
    FLY_CUDA(cudaMemcpyAsync(hess, H.p, sizeof(double) * N * N, cudaMemcpyDeviceToHost, list->stream));
    FLY_CUDA(cudaStreamSynchronize(list->stream));
    release_large_hessian(list);
  });
}

int flygpu_hessian_eigenvalues(flygpu_eam* eam, flygpu_list* list, const uint32_t* types, const uint8_t* frozen,
                               const double* masses, double* eig, double* hess) {
  return guard([&] {
    need(eam && list && eig, "null argument");
    need(list->built, "EAM call before List::rebuild()");
    need(types && frozen, "types and frozen flags are required");
    list_set_atoms(list, eam->n_types, nullptr, nullptr, true, types, frozen);
    hessian_prefactor_one(eam, list, types, frozen, masses, eig, hess);
    release_large_hessian(list);
  });
}

int flygpu_hessian_eigenvalues_batch(flygpu_eam* eam, const flygpu_search_desc* systems, int n_systems,
                                     const double* masses, int workers, double* eig) {
  return guard([&] {
    need(eam && eig && (systems || n_systems == 0), "null argument");
    need(n_systems >= 0, "negative system count");
    if (n_systems == 0) return;
    std::vector<std::size_t> off(static_cast<std::size_t>(n_systems) + 1, 0);
    for (int k = 0; k < n_systems; ++k) {
      need(systems[k].n >= 0 && (systems[k].n == 0 || (systems[k].pos && systems[k].types && systems[k].frozen)),
           "each system needs positions, types and frozen flags");
      off[static_cast<std::size_t>(k) + 1] = off[static_cast<std::size_t>(k)] + 3 * static_cast<std::size_t>(systems[k].n);
    }
    int const P = std::max(1, std::min(workers > 0 ? workers : 8, n_systems));
    std::vector<int> status(static_cast<std::size_t>(n_systems), FLYGPU_OK);
    std::vector<std::string> msg(static_cast<std::size_t>(n_systems));
    int dev = 0;
    FLY_CUDA(cudaGetDevice(&dev));
    auto work = [&](int w) {
      // worker w: systems w, w + P, ... on its own stream and list (with its scratch); every CUDA call sits
      // inside guard (an exception must not leave the thread)
      std::unique_ptr<flygpu_list> L;
      for (int k = w; k < n_systems; k += P) {
        flygpu_search_desc const& d = systems[k];
        int const st = guard([&] {
          FLY_CUDA(cudaSetDevice(dev));
          if (!L) {
            L = std::make_unique<flygpu_list>();
            FLY_CUDA(cudaStreamCreateWithFlags(&L->stream, cudaStreamNonBlocking));
            L->own_stream = true;
            L->err.reserve(1);
            L->counters.reserve(8);
            L->h_small.reserve(8);
            FLY_CUDA(cudaMemsetAsync(L->err.p, 0, sizeof(int), L->stream));
          }
          list_set_box(L.get(), d.extents, d.periodic, eam->r_cut);
          if (d.n > 0) {
            L->io.reserve(3 * static_cast<std::size_t>(d.n) + 3);
            FLY_CUDA(cudaMemcpyAsync(L->io.p, d.pos, sizeof(double) * 3 * static_cast<std::size_t>(d.n),
                                     cudaMemcpyHostToDevice, L->stream));
          }
          list_rebuild(L.get(), L->io.p, d.n);
          check_device(L.get());
          list_set_atoms(L.get(), eam->n_types, nullptr, nullptr, true, d.types, d.frozen);
          if (d.n > 0) hessian_prefactor_one(eam, L.get(), d.types, d.frozen, masses, eig + off[static_cast<std::size_t>(k)], nullptr);
        });
        status[static_cast<std::size_t>(k)] = st;
        if (st != FLYGPU_OK) msg[static_cast<std::size_t>(k)] = flygpu_last_error();
      }
      if (L) {
        cudaStreamSynchronize(L->stream);
        cudaStream_t const s = L->stream;
        L.reset();
        cudaStreamDestroy(s);
      }
    };
    std::vector<std::thread> th;
    for (int w = 1; w < P; ++w) th.emplace_back(work, w);
    work(0);
    for (auto& t : th) t.join();
    for (int k = 0; k < n_systems; ++k)
      if (status[static_cast<std::size_t>(k)] != FLYGPU_OK)
        fail(status[static_cast<std::size_t>(k)], "system " + std::to_string(k) + ": " + msg[static_cast<std::size_t>(k)]);
  });
}

int flygpu_eam_energy_gradient_device(flygpu_eam* eam, flygpu_list* list, const uint32_t* d_types,
                                      const uint8_t* d_frozen, int precision, double* d_energy, double* d_grad) {
  return guard([&] {
    need(eam && list, "null handle");
    need(list->built, "EAM call before List::rebuild()");
    if (d_types || d_frozen || !list->types_set) list_set_atoms(list, eam->n_types, d_types, d_frozen, false, nullptr, nullptr);
    run_eam(eam, list, precision, d_energy, d_grad);
  });
}

}  // extern "C"
