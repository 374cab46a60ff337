// search.cu -- host side of the batched search kernel: device-block layout of one search, binding,
// output gather and the choice among the kernel variants (search_kernel.cuh; one translation unit per
// precision and lanes-per-atom, search_{m,d}{1,2,4,8}.cu).

#include <mutex>

#include <algorithm>

#include "search.hpp"

namespace flygpu {

  namespace {

    SearchKernels kernels(bool mixed, int lpa) {
      switch (lpa) {
        case 1: return mixed ? search_kernels<true, 1>() : search_kernels<false, 1>();
        case 2: return mixed ? search_kernels<true, 2>() : search_kernels<false, 2>();
        case 4: return mixed ? search_kernels<true, 4>() : search_kernels<false, 4>();
        case 8: return mixed ? search_kernels<true, 8>() : search_kernels<false, 8>();
        default: fail(FLYGPU_INVALID_ARG, "lanes per atom must be 1, 2, 4 or 8");
      }
    }

    // max_registers 0: the compiler's allocation; 128: the capped variant.
    SearchKernel pick(bool mixed, int lpa, int max_registers) {
      if (max_registers != 0 && max_registers != 128) fail(FLYGPU_INVALID_ARG, "max_registers must be 0 or 128");
      return kernels(mixed, lpa).k[max_registers == 128 ? 1 : 0];
    }

    // Mobile positions and axes of every search into compact arrays (3 per mobile atom, batch order).
    __global__ void k_gather_out(BatchView bv, std::int64_t const* __restrict__ act3, double* __restrict__ ox,
                                 double* __restrict__ oa) {
      int const s = blockIdx.x;
      if (s >= bv.n_search) return;
      SearchDev const& S = bv.S[s];
      int const M = 3 * S.na;
      double const* v = S.vec;
      std::int64_t const o = act3[s];
      for (int e = threadIdx.x; e < M; e += blockDim.x) {
        ox[o + e] = v[static_cast<std::int64_t>(V_X) * M + e];
        oa[o + e] = S.mode == MODE_DIMER ? v[static_cast<std::int64_t>(V_AX) * M + e] : 0.0;
      }
    }

    // Ordered compaction of the unfinished items (one CTA of 1024 threads, ballot prefix sums).
    __global__ void k_unfinished(SearchDev const* __restrict__ S, int const* __restrict__ order, int n,
                                 int* __restrict__ out, int* __restrict__ n_out) {
      __shared__ int base;
      __shared__ int wcount[32];
      int const lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
      if (threadIdx.x == 0) base = 0;
      __syncthreads();
      for (int k0 = 0; k0 < n; k0 += blockDim.x) {
        int const k = k0 + threadIdx.x;
        bool const keep = k < n && S[order[k]].stage != STAGE_DONE;
        unsigned const bal = __ballot_sync(0xffffffffu, keep);
        if (lane == 0) wcount[w] = __popc(bal);
        __syncthreads();
        int off = base;
        for (int q = 0; q < w; ++q) off += wcount[q];
        if (keep) out[off + __popc(bal & ((1u << lane) - 1u))] = order[k];
        __syncthreads();
        if (threadIdx.x == 0) {
          int t = 0;
          for (int q = 0; q < nw; ++q) t += wcount[q];
          base += t;
        }
        __syncthreads();
      }
      if (threadIdx.x == 0) *n_out = base;
    }

  }  // namespace

  void search_unfinished(SearchDev const* S, int const* order, int n, int* order_out, int* n_out, cudaStream_t s) {
    launch(k_unfinished, 1, 1024, 0, s, S, order, n, order_out, n_out);
  }

  namespace {
    __global__ void k_image_scatter(char* __restrict__ block, char const* __restrict__ src,
                                    ImageChunk const* __restrict__ ch, int n) {
      int const w = static_cast<int>((static_cast<long long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5);
      int const lane = threadIdx.x & 31;
      if (w >= n) return;
      ImageChunk const c = ch[w];
      long long const words = c.bytes / 8;
      auto* d8 = reinterpret_cast<unsigned long long*>(block + c.dst);
      auto const* s8 = reinterpret_cast<unsigned long long const*>(src + c.src);
      for (long long i = lane; i < words; i += 32) d8[i] = s8[i];
      for (long long i = words * 8 + lane; i < c.bytes; i += 32) block[c.dst + i] = src[c.src + i];
    }
  }  // namespace

  void search_image_scatter(char* block, char const* d_src, ImageChunk const* d_chunks, int n, cudaStream_t s) {
    if (n > 0) launch(k_image_scatter, static_cast<unsigned>((n + 7) / 8), 256, 0, s, block, d_src, d_chunks, n);
  }

  SearchLayout search_layout(int n, int na, int n_vec_doubles, int n_hist_doubles) {
    auto up = [](std::size_t b) { return (b + 255) / 256 * 256; };
    SearchLayout l{};
    std::size_t o = 0;
    l.xl = o;
    o += up(sizeof(D4) * static_cast<std::size_t>(n));
    l.pk = o;
    o += up(sizeof(Packed) * static_cast<std::size_t>(n));
    l.vec = o;
    o += up(sizeof(double) * static_cast<std::size_t>(n_vec_doubles));
    l.hist = o;
    o += up(sizeof(double) * static_cast<std::size_t>(n_hist_doubles));
    l.aatom = o;
    o += up(sizeof(int) * static_cast<std::size_t>(na));
    l.nbr = o;
    o += up(sizeof(std::uint16_t) * static_cast<std::size_t>(n) * NB_CAP);
    l.ncnt = o;
    o += up(sizeof(std::uint16_t) * static_cast<std::size_t>(n));
    l.type = o;
    o += up(static_cast<std::size_t>(n));
    l.mob = o;
    o += up(static_cast<std::size_t>(n));
    l.rho0 = o;
    o += up(sizeof(double) * static_cast<std::size_t>(n));
    l.need = o;
    o += up(sizeof(std::uint16_t) * static_cast<std::size_t>(n));
    l.mark = o;
    o += up(sizeof(int) * static_cast<std::size_t>(n));
    l.dacc = o;
    o += up(sizeof(long long) * static_cast<std::size_t>(n));
    l.total = o;
    return l;
  }

  void search_bind(SearchDev& S, char* base, SearchLayout const& l) {
    S.xl = reinterpret_cast<D4*>(base + l.xl);
    S.pk = reinterpret_cast<Packed*>(base + l.pk);
    S.type = reinterpret_cast<std::uint8_t*>(base + l.type);
    S.aatom = reinterpret_cast<int*>(base + l.aatom);
    S.ncnt = reinterpret_cast<std::uint16_t*>(base + l.ncnt);
    S.nbr = reinterpret_cast<std::uint16_t*>(base + l.nbr);
    S.vec = reinterpret_cast<double*>(base + l.vec);
    S.hist = reinterpret_cast<double const*>(base + l.hist);
    S.mob = reinterpret_cast<std::uint8_t*>(base + l.mob);
    S.rho0 = reinterpret_cast<double*>(base + l.rho0);
    S.need = reinterpret_cast<std::uint16_t*>(base + l.need);
    S.mark = reinterpret_cast<int*>(base + l.mark);
    S.dacc = reinterpret_cast<long long*>(base + l.dacc);
  }

  void search_gather(BatchView const& v, std::int64_t const* d_act3_off, double* out_x, double* out_ax,
                     cudaStream_t s) {
    launch(k_gather_out, v.n_search, 128, 0, s, v, d_act3_off, out_x, out_ax);
  }

  // The search kernels' shared-memory limit is a property of the current context (a device reset drops
  // it), so it is set again before every occupancy query and every launch outside a stream capture, always
  // to the same constant (concurrent host threads agree); a capture relies on search_init_kernels() having
  // run just before it.
  namespace {
    void set_smem_cap(SearchKernel k) {
      FLY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, SEARCH_SMEM_CAP));
    }
  }  // namespace

  void search_init_kernels() {
    for (bool mixed : {true, false})
      for (int lpa : {1, 2, 4, 8})
        for (SearchKernel k : kernels(mixed, lpa).k) set_smem_cap(k);
  }

  void search_occupancy(int lanes_per_atom, int threads, bool mixed, int max_registers, int smem_bytes,
                        int* blocks_per_sm) {
    SearchKernel const k = pick(mixed, lanes_per_atom, max_registers);
    set_smem_cap(k);
    FLY_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm, k, threads, static_cast<std::size_t>(smem_bytes)));
  }

  int search_smem_for(int lanes_per_atom, int threads, bool mixed, int max_registers, int blocks_per_sm, int need) {
    int bps = 0;
    search_occupancy(lanes_per_atom, threads, mixed, max_registers, need, &bps);
    if (bps >= blocks_per_sm) return need;
    int dev = 0, per_sm = 0;
    FLY_CUDA(cudaGetDevice(&dev));
    FLY_CUDA(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
    // start from an even split of the SM's shared memory and step down by 1 KB
    for (int b = std::min(need, per_sm / std::max(1, blocks_per_sm)) / 1024 * 1024; b >= 0; b -= 1024) {
      search_occupancy(lanes_per_atom, threads, mixed, max_registers, b, &bps);
      if (bps >= blocks_per_sm) return b;
    }
    return 0;
  }

  void search_launch(BatchView const& v, int lanes_per_atom, int threads, int max_registers, int blocks, bool mixed,
                     cudaStream_t s) {
    if (threads % 32 != 0 || threads < 64 || threads > 1024)
      fail(FLYGPU_INVALID_ARG, "threads must be 64..1024, a multiple of 32");
    if (v.smem_bytes < 0 || v.smem_bytes > SEARCH_SMEM_CAP) fail(FLYGPU_INVALID_ARG, "search shared memory out of range");
    SearchKernel const k = pick(mixed, lanes_per_atom, max_registers);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    FLY_CUDA(cudaStreamIsCapturing(s, &cap));
    if (cap == cudaStreamCaptureStatusNone) set_smem_cap(k);
    launch(k, blocks, threads, static_cast<std::size_t>(v.smem_bytes), s, v);
  }

}  // namespace flygpu
