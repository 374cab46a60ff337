// internal.hpp -- structures shared by the host and device translation units of libflygpu.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/flygpu.h"

namespace flygpu {

  // 32-byte aligned binary64 quadruple: a position (+ one scalar) or a spline interval {a, b, c, d};
  // one 32-byte sector per access.
  struct alignas(32) D4 {
    double x, y, z, w;
  };

  // ------------------------------------------------------------------ errors

  void set_error(std::string msg);

  struct Error {
    int status;
    std::string msg;
  };

  [[noreturn]] void fail(int status, std::string msg);

  inline void cuda_check(cudaError_t e, char const* what) {
    if (e == cudaErrorMemoryAllocation) fail(FLYGPU_OOM, std::string(what) + ": " + cudaGetErrorString(e));
    if (e != cudaSuccess) fail(FLYGPU_CUDA_ERROR, std::string(what) + ": " + cudaGetErrorString(e));
  }

#define FLY_CUDA(call) ::flygpu::cuda_check((call), #call)

  // Device-side error word bits (one word per list handle). Kernels never trap: they set a bit and
  // skip the offending access; the host turns the word into a status after the next sync.
  enum : int {
    ERR_SPLINE_OOB = 1,
    ERR_NLIST_OVERFLOW = 2,
    ERR_GHOST_OVERFLOW = 4,
    ERR_BAD_INDEX = 8,
    ERR_TIMEOUT = 16,
  };

  int status_from_word(int word);

  // ------------------------------------------------------------------ launches

  // Kernel launches made by this library since load (all go through launch()).
  void count_launch();
  long long launch_count();

#ifdef __CUDACC__
  template <typename... KArgs, typename... Args>
  inline void launch(void (*k)(KArgs...), dim3 grid, dim3 block, std::size_t smem, cudaStream_t s, Args&&... args) {
    k<<<grid, block, smem, s>>>(static_cast<KArgs>(args)...);
    count_launch();
    cuda_check(cudaGetLastError(), "kernel launch");
  }
#endif

  // ------------------------------------------------------------------ device buffers

  template <typename T>
  struct DevBuf {
    T* p = nullptr;
    std::size_t n = 0;

    DevBuf() = default;
    DevBuf(DevBuf const&) = delete;
    DevBuf& operator=(DevBuf const&) = delete;
    ~DevBuf() { release(); }

    void release() {
      if (p) cudaFree(p);
      p = nullptr;
      n = 0;
    }
    // Grow to at least count elements; contents are not preserved.
    void reserve(std::size_t count) {
      if (count <= n) return;
      release();
      std::size_t want = count + count / 8 + 16;
      FLY_CUDA(cudaMalloc(&p, want * sizeof(T)));
      n = want;
    }
    // Grow to at least count elements keeping the first keep elements.
    void grow_keep(std::size_t count, std::size_t keep, cudaStream_t s) {
      if (count <= n) return;
      T* q = nullptr;
      std::size_t want = count + count / 4 + 16;
      FLY_CUDA(cudaMalloc(&q, want * sizeof(T)));
      if (p && keep) FLY_CUDA(cudaMemcpyAsync(q, p, keep * sizeof(T), cudaMemcpyDeviceToDevice, s));
      FLY_CUDA(cudaStreamSynchronize(s));
      if (p) cudaFree(p);
      p = q;
      n = want;
    }
  };

  template <typename T>
  struct PinnedBuf {
    T* p = nullptr;
    std::size_t n = 0;
    PinnedBuf() = default;
    PinnedBuf(PinnedBuf const&) = delete;
    PinnedBuf& operator=(PinnedBuf const&) = delete;
    ~PinnedBuf() {
      if (p) cudaFreeHost(p);
    }
    void reserve(std::size_t count) {
      if (count <= n) return;
      if (p) cudaFreeHost(p);
      p = nullptr;
      FLY_CUDA(cudaMallocHost(&p, count * sizeof(T)));
      n = count;
    }
  };

  // ------------------------------------------------------------------ EAM tables

  // Per function kind the device holds binary64 {a,b,c,d} per interval (reference form) and binary32
  // coefficients of the same cubic in the interval's unit coordinate t = x/dx - i:
  // f = a + t(b' + t(c' + t d')) with b' = b dx, c' = c dx^2, d' = d dx^3.
  struct SplineSet {
    int count = 0;        // number of functions of this kind
    int n_spines = 0;     // intervals per function
    double dx = 0, inv_dx = 0;
    std::vector<double> host;  // count * n_spines * 4
    DevBuf<D4> d64;
    DevBuf<float4> d32;
  };

  // Merged binary32 spline record of one (receiver type t_i, neighbour type t_n, interval): phi of the
  // neighbour's type at the receiver (phi_{t_n -> t_i}, the reference's phi[t_n + n t_i]) and the pair
  // potential v_{t_i t_n}, both in the interval's unit coordinate. 32 bytes: one sector, one 256-bit load.
  struct alignas(32) PairRec {
    float4 phi, v;
  };

  // Derivative record of the same (t_i, t_n, interval) for the binary32 force pass: v_{t_i t_n} and
  // phi_{t_n -> t_i} as {b_hi, b_lo, 2c, 3d} in the unit coordinate (b = b_hi + b_lo to ~2^-48, so
  // df/dt = b_hi + (b_lo + t (2c + 3 t d)) carries no rounding of its leading coefficient).
  struct alignas(32) DerRec {
    float4 v, phi;
  };

  // Device view passed to kernels by value.
  struct TablesView {
    int n_types;
    int nP, nR;  // intervals of F and of phi / v
    double dP, inv_dP, dR, inv_dR;
    float fdP, finv_dP, fdR, finv_dR;
    float finv_dR_lo;  // 1/dR - finv_dR: 1/dR as a binary32 pair
    D4 const* F64;
    D4 const* phi64;  // [a + n*b] * nR
    D4 const* v64;    // both orders filled
    float4 const* F32;
    float4 const* phi32;
    float4 const* v32;
    PairRec const* pv32;  // [t_i * n_types + t_n] * nR + interval
    DerRec const* dv32;   // same indexing
  };

}  // namespace flygpu

struct flygpu_eam {
  int n_types = 0;
  double r_cut = 0;
  std::vector<std::string> names;
  std::vector<double> mass;
  flygpu::SplineSet F, phi, v;  // phi and v hold n*n functions (v symmetric, both orders)
  flygpu::DevBuf<flygpu::PairRec> pv;  // phi and v of each ordered type pair merged per interval
  flygpu::DevBuf<flygpu::DerRec> dv;   // their derivative records
  flygpu::TablesView view() const;
};

namespace flygpu {

  struct GridDesc {
    double L[3];
    double cell[3], inv_cell[3];
    int shape[3];
    int per[3];
    double rc;  // list cut-off
    int ncells() const { return shape[0] * shape[1] * shape[2]; }
  };

  // Binary32 slot record for the MIXED passes: the position as (hi, lo) pairs of an offset coordinate
  // x + shift whose hi parts all lie in one binade, so hi differences are exact; plus the slot's type
  // and its atom's F'(rho). 32 bytes, one sector per neighbour gather.
  struct alignas(32) Packed {
    float hx, hy, hz;
    std::uint32_t type;
    float lx, ly, lz;
    float fp;
  };

  // Device scratch of the Hessian calls, kept by the list handle so repeated calls allocate nothing (a
  // cudaFree would synchronise the whole device and serialise concurrent callers).
  struct HessianScratch {
    DevBuf<long long> offs;
    DevBuf<int> idx, act, cols, key;
    DevBuf<double> dr, rho_mu, fder, pr, pfp, m3, sub, H, tri;
    DevBuf<std::uint32_t> ty;
  };

  // Largest matrix the dense eigensolver takes (three vectors of this many doubles in shared memory).
  constexpr int MAX_DENSE_EIG = 9000;

}  // namespace flygpu

struct flygpu_list {
  flygpu::GridDesc g{};
  double shift[3] = {0, 0, 0};  // offset of the binary32 packed coordinates
  cudaStream_t stream = nullptr;
  bool own_stream = false;

  std::int64_t n = 0;        // real atoms
  std::int64_t n_slots = 0;  // real + ghost
  int nb_cap = 0;            // neighbour capacity per atom
  bool built = false;

  // reference-order slots (real atoms then ghosts in List::make_ghosts order)
  flygpu::DevBuf<flygpu::D4> r_ref;
  flygpu::DevBuf<int> img_ref, cell_ref, flag_p, flag_m, scan_p, scan_m;
  // physical (cell-sorted) slots
  flygpu::DevBuf<flygpu::D4> pos;   // xyz + w = F'(rho) of the slot's atom (FP64 passes)
  flygpu::DevBuf<int> pimg;      // real index of each physical slot
  flygpu::DevBuf<int> pref;      // reference slot id of each physical slot
  flygpu::DevBuf<int> ptype;     // type of each physical slot
  flygpu::DevBuf<flygpu::Packed> packed;
  flygpu::DevBuf<float4> hi;     // binary32 hi parts of the offset coordinates (build prefilter)
  flygpu::DevBuf<int> cell_count, cell_start, cell_fill, members;
  flygpu::DevBuf<int> real_phys;  // physical slot of the j-th real atom in cell order
  flygpu::DevBuf<int> nbr;        // [nb_cap][n] physical neighbour slots, column per atom
  flygpu::DevBuf<int> ncount;
  // per real atom
  flygpu::DevBuf<std::uint32_t> types;
  flygpu::DevBuf<std::uint8_t> frozen;
  flygpu::DevBuf<double> fprime;   // F'(rho) by real index
  flygpu::DevBuf<double> io;       // 3n staging for host copies
  flygpu::DevBuf<double> energy_part;
  flygpu::DevBuf<double> energy;   // 1
  flygpu::DevBuf<int> scan_tmp;
  flygpu::DevBuf<int> err;         // device error word
  flygpu::DevBuf<int> counters;    // small device counters
  flygpu::PinnedBuf<int> h_small;  // pinned mirror of counters / error word
  flygpu::PinnedBuf<double> h_io;
  bool types_set = false;
  bool frozen_set = false;
  bool packed_valid = false;
  // CUDA-event timing of the main kernels (enabled by flygpu_list_set_timing)
  bool timing = false;
  flygpu::HessianScratch hs;
  flygpu::DevBuf<int> export_counts;  // per-atom counts of list_export_device
  std::vector<cudaEvent_t> ev_pool;
  std::size_t ev_used = 0;
  struct Mark {
    int kind;
    cudaEvent_t a, b;
  };
  std::vector<Mark> marks;
  ~flygpu_list() {
    for (cudaEvent_t e : ev_pool) cudaEventDestroy(e);
  }
};

namespace flygpu {

  // nlist.cu
  void list_rebuild(flygpu_list* L, double const* d_pos, std::int64_t n);
  void list_update(flygpu_list* L, double const* d_delta);
  // For each real atom (reference index) its neighbours within r_cut in the list's order, on the device:
  // offs[i] = first entry of atom i (n + 1 entries, offs[n] = the total), idx (reference indices) and dr
  // (xyz, binary64 r_n - r_i). Returns the per-atom counts on the host: waits for the counting pass; the
  // filling pass runs on after the return, on the list's stream.
  std::vector<int> list_export_device(flygpu_list* L, double r_cut, DevBuf<long long>& offs, DevBuf<int>& idx,
                                      DevBuf<double>& dr);
  // One real atom's neighbours within r_cut in List::for_neighbours order: real indices and binary64
  // r_n - r_i (3 per entry). Synchronises the list's stream; returns the count.
  int list_neighbours_of(flygpu_list* L, double r_cut, std::int64_t atom, std::vector<int>& idx,
                         std::vector<double>& dr);
  // n_types bounds the type indices (out-of-range types raise FLYGPU_INVALID_ARG).
  void list_set_atoms(flygpu_list* L, int n_types, std::uint32_t const* d_types, std::uint8_t const* d_frozen,
                      bool copy_from_host, std::uint32_t const* h_types, std::uint8_t const* h_frozen);
  void list_pack(flygpu_list* L);
  int list_take_error(flygpu_list* L);  // syncs, reads and clears the device error word
  std::int64_t list_export(flygpu_list* L, double r_cut, int* counts, int* idx, double* dr, std::int64_t cap);
  void exclusive_scan(int const* in, int* out, std::int64_t n, int* tmp, std::size_t tmp_len, cudaStream_t s);
  std::size_t scan_tmp_size(std::int64_t n);

  // Kernel timing kinds recorded by the list handle.
  enum : int { TK_DENSITY = 0, TK_FORCE = 1, TK_UPDATE = 2, TK_REBUILD = 3, TK_COUNT = 4 };
  // Records an event on the list's stream when timing is on (returns nullptr otherwise).
  cudaEvent_t timer_record(flygpu_list* L);
  void timer_mark(flygpu_list* L, int kind, cudaEvent_t a, cudaEvent_t b);

  // eam_fp64.cu / eam_mixed.cu
  void eam_fp64(flygpu_eam const* E, flygpu_list* L, double* d_energy, double* d_grad);
  void eam_mixed(flygpu_eam const* E, flygpu_list* L, double* d_energy, double* d_grad);

  // hessian.cu: the dense 3n x 3n EAM Hessian into d_H (row-major, lower blocks); its mass weighting
  // (type_mass per type, NULL for the potential file's masses); the ascending eigenvalues of a symmetric
  // matrix given by its row-major lower triangle (d_H is overwritten). Each synchronises the stream and
  // keeps its scratch in L->hs.
  void eam_hessian(flygpu_eam const* E, flygpu_list* L, std::uint8_t const* h_frozen, double* d_H);
  void hessian_mass_weight(flygpu_eam const* E, flygpu_list* L, double const* type_mass, std::uint32_t const* h_types,
                           double* d_H);
  // eigen.cu: ascending eigenvalues of the symmetric matrix given by the row-major lower triangle of the
  // N x N d_H, restricted to the coordinates `act` (all of them when act is empty); d_H is not modified.
  void dense_eigenvalues(flygpu_list* L, double const* d_H, std::int64_t N, std::vector<int> const& act, double* h_eig);
  // The same for a 3n x 3n Hessian whose frozen atoms' rows and columns are zero (only the active block
  // is diagonalised; one exact zero per frozen coordinate is merged in).
  void hessian_eigenvalues(flygpu_list* L, double* d_H, std::uint8_t const* h_frozen, double* h_eig);

  // perturb.cpp: Master::perturb given the centre's neighbours (real indices and distances, in
  // List::for_neighbours order); returns the stddev drawn.
  double perturb(std::vector<int> const& nbr, std::vector<double> const& nbr_r, std::int64_t centre,
                 double const* in_pos, std::uint8_t const* frozen, std::int64_t n, double stddev_opt, double r_pert,
                 flygpu_xoshiro& g, double* out_pos, double* out_axis);

  // tables.cpp
  void build_spline(std::vector<double> y, double dx, double* out4, int n_spines);
  int spline_spines(std::size_t n_samples);

}  // namespace flygpu
