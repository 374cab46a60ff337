// search.hpp -- device data layout of batched, resumable dimer searches and L-BFGS minimisations.
#pragma once

#include <cstdint>
#include <vector>

#include "internal.hpp"

namespace flygpu {

  constexpr int NB_CAP = 96;       // neighbour capacity per atom inside a search (uint16 local indices)
  constexpr int MAX_ATOMS = 4096;  // atoms per search (local indices fit in uint16 with room to spare)
  constexpr int MAX_HIST = 16;     // L-BFGS history length supported on the device
  constexpr int N_VEC = 15;        // fixed per-DOF vectors of a search (see Vec below)
  // Dynamic shared memory a CTA may use to stage the search it runs (vectors, positions, slot records):
  // two CTAs of this size fit in one SM's 228 KB.
  constexpr int SEARCH_SMEM_CAP = 100 * 1024;

  // Bytes of the shared-memory image of a search of n atoms whose vectors hold n_vec_doubles doubles:
  // vectors (rounded to 128 B), then positions (D4), then binary32 slot records.
  inline std::size_t search_smem_need(int n, std::size_t n_vec_doubles) {
    std::size_t const vb = (n_vec_doubles * sizeof(double) + 127) / 128 * 128;
    return vb + static_cast<std::size_t>(n) * (sizeof(D4) + sizeof(Packed));
  }

  enum Mode : int { MODE_DIMER = 0, MODE_MINIMISE = 1 };
  enum Stage : int { STAGE_INIT = 0, STAGE_LOOP = 1, STAGE_DONE = 2 };

  // Per-DOF vectors (3 doubles per mobile atom), in this order inside a search's vector block.
  enum Vec : int {
    V_X = 0,      // dimer / minimiser positions of mobile atoms (Position)
    V_AX,         // dimer axis (Axis)
    V_EFF,        // effective gradient (dimer) or gradient (minimiser)
    V_G0,         // rotor: gradient at the centre
    V_G1,         // rotor: gradient at the end
    V_G1P,        // rotor: gradient at the trial end
    V_DPREV,      // rotor: displacement currently applied to the list
    V_AXP,        // rotor: trial axis
    V_TH,         // rotor L-BFGS output (rotation plane)
    V_HG,         // translation L-BFGS output (step)
    V_PXT, V_PGT, // translation L-BFGS previous x / g
    V_PXR, V_PGR, // rotation L-BFGS previous x / g
    V_INMIN,      // minimum the dimer climbs from (history check)
  };

  // Options shared by every search of a batch (Dimer::Options dimer.hpp:56-98, Rotor::Options
  // rotor.hpp:47-60, LBFGS::Options lbfgs.hpp:56-80).
  struct SearchOpts {
    int mT, max_steps, hist_check_freq, use_history;
    double f2norm, skin_frac, proj_tol, max_trust, min_trust, grow_trust, shrink_trust, convex_max;
    int mR, iter_max_rot, relax_in_convex;
    double delta_r, theta_tol;
    // L-BFGS minimiser
    int mL, iter_max_l;
    double f2norm_l, skin_frac_l, proj_tol_l, max_trust_l, min_trust_l, grow_trust_l, shrink_trust_l;
    double r_cut;  // potential cut-off
  };

  // One search: geometry, offsets into the batch arrays, resumable scalar state and results.
  struct SearchDev {
    int n, na, mode, count_frozen;
    int n_hist, stage, it, kT;
    int exit_code, status, pad0, pad1;
    double L[3];
    int per[3], periodic_any;
    double shift[3];        // binary32 packed-coordinate offset per axis
    double rc_list;         // neighbour-list cut-off of this search
    double theta_tol_hist;  // collision angle (Master::find_batch, find.cpp:692)
    // |x - in_min|^2 over the static atoms (fixed for the search): with the per-saddle sums stored after
    // the history vectors it makes the device's mobile-DOF history check the reference's 3N one
    double hist_static_on2;
    // this search's arrays (inside a batch's shared buffers or a served request's own block)
    D4* xl;                 // list positions per atom (w = F')
    Packed* pk;             // binary32 records per atom
    std::uint8_t* type;     // per atom
    int* aatom;             // per mobile atom: local atom index
    std::uint16_t* ncnt;    // per atom
    std::uint16_t* nbr;     // [NB_CAP][n]
    double* vec;            // (N_VEC + 2 mT + 2 mR) vectors of 3 na doubles
    double const* hist;     // n_hist vectors of 3 na doubles (previous saddle points), then per saddle h
                            // sum (x - in_min).(sp_h - in_min) and |sp_h - in_min|^2 over static atoms
    std::uint8_t* mob;      // per atom: 1 if it can move (mobile), else 0
    double* rho0;           // per static atom: density from its static neighbours (fixed for the search)
    std::uint16_t* need;    // atoms whose F' the force pass reads (mobile atoms and their neighbours)
    int* mark;              // per atom: scratch flag of the needed-list build
    long long* dacc;        // per atom: its mobile neighbours' density terms in fixed point (L2 atomics)
    int n_need, pad2;
    double trust, acc, convex, curv, energy;
    std::int64_t grad_calls;
    double rhoT[MAX_HIST], alphaT[MAX_HIST];
  };

  struct BatchView {
    SearchDev* S;
    int n_search;
    int const* order;         // work items -> search index
    int n_items;
    int const* n_items_dev;   // if set, the item count is read from device memory (graph replays)
    int* work;                // atomic work counter
    int budget;               // translation steps per launch (<= 0: run to completion)
    int smem_bytes;           // dynamic shared memory per CTA for staging a search's state (0: none)
    SearchOpts o;
    TablesView tb;
  };

  // Byte offsets of one search's arrays inside its block (256-byte aligned parts).
  struct SearchLayout {
    std::size_t xl, pk, type, aatom, ncnt, nbr, vec, hist, mob, rho0, need, mark, dacc, total;
  };

  // search_{m,d}{1,2,4,8}.cu: the kernel variants of one precision and lanes-per-atom.
  using SearchKernel = void (*)(BatchView);
  struct SearchKernels {
    SearchKernel k[2];  // [0] the compiler's register allocation, [1] at most 128 registers a thread
  };
  template <bool MIXED, int LPA>
  SearchKernels search_kernels();
  template <> SearchKernels search_kernels<true, 1>();
  template <> SearchKernels search_kernels<true, 2>();
  template <> SearchKernels search_kernels<true, 4>();
  template <> SearchKernels search_kernels<true, 8>();
  template <> SearchKernels search_kernels<false, 1>();
  template <> SearchKernels search_kernels<false, 2>();
  template <> SearchKernels search_kernels<false, 4>();
  template <> SearchKernels search_kernels<false, 8>();

  // search.cu
  void search_launch(BatchView const& v, int lanes_per_atom, int threads, int max_registers, int blocks, bool mixed,
                     cudaStream_t s);
  void search_occupancy(int lanes_per_atom, int threads, bool mixed, int max_registers, int smem_bytes,
                        int* blocks_per_sm);
  // The largest staging budget (dynamic shared memory per CTA, at most need) at which blocks_per_sm CTAs
  // of the shape stay resident on one SM; 0 when even no staging does not allow that many.
  int search_smem_for(int lanes_per_atom, int threads, bool mixed, int max_registers, int blocks_per_sm, int need);
  // Lets every kernel variant use SEARCH_SMEM_CAP bytes of dynamic shared memory (once per process;
  // call before any graph capture).
  void search_init_kernels();
  SearchLayout search_layout(int n, int na, int n_vec_doubles, int n_hist_doubles);
  // A region of a search image written on the host: `bytes` bytes from `src` of a compact host buffer to
  // byte `dst` of the device block. The rest of a block starts as zeros.
  struct ImageChunk {
    long long dst, src, bytes;
  };
  // Copies n chunks from d_src into the (zeroed) block on stream s, one warp per chunk; dst and src are
  // 8-byte aligned.
  void search_image_scatter(char* block, char const* d_src, ImageChunk const* d_chunks, int n, cudaStream_t s);
  void search_bind(SearchDev& S, char* base, SearchLayout const& l);
  // The items of order[0..n) whose search has not finished, in the same order, into order_out, and
  // their count into *n_out (device memory). One CTA.
  void search_unfinished(SearchDev const* S, int const* order, int n, int* order_out, int* n_out, cudaStream_t s);

  // search_host.cpp: fill one search's state and initial arrays (image at byte `at` of img; a grown img
  // is zero-filled, a reused one keeps its old bytes outside the regions search_written writes).
  SearchLayout search_prepare(SearchOpts const& o, int n_types, flygpu_search_desc const& d, SearchDev& S,
                              std::vector<int>& mob, std::vector<char>& img, std::size_t at);
  // The (offset, bytes) regions of a search image that search_prepare writes; every other byte of the
  // image is zero.
  std::vector<std::pair<std::size_t, std::size_t>> search_written(SearchLayout const& l, SearchDev const& S);
  SearchOpts make_opts(flygpu_dimer_options const& d, flygpu_lbfgs_options const& l, double r_cut);

}  // namespace flygpu
