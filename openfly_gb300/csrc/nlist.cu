// nlist.cu -- neighbour-list rebuild / update on the GPU (compiled with -fmad=false).
//
// Restates neigh::List (src/neigh/list.cpp:37-165) for an orthorhombic box:
//   1. real atoms -> canonical images            (list.cpp:68-72, orthorhombic.hpp:132-139)
//   2. ghosts axis by axis, plus then minus pass  (list.cpp:100-132, orthorhombic.hpp:54-74)
//   3. linked cells                               (list.cpp:84-89, hypergrid.hpp:75-99)
//   4. per-atom lists: own cell then adjacent cells in increasing index (adjacent.hpp:40-70),
//      each cell newest-inserted first (head insertion), r^2 < rc^2   (list.cpp:134-165)
// GB300 layout: slots are generated in the reference's order (so ghost numbering is identical), then
// counting-sorted by cell into a physical order whose within-cell order is ascending reference slot.
// Walking a cell from its last physical slot to its first is then exactly the reference's
// linked-list order, so every atom's neighbour sequence -- and every binary64 sum over it -- matches
// the reference. Positions are D4 (one 32-byte sector per gather); neighbour lists are stored
// column-per-atom ([k][j]) so a warp's loads of the k-th neighbour are coalesced.

#include <algorithm>
#include <cmath>

#include "internal.hpp"

namespace flygpu {

  namespace {

    constexpr int T = 256;

    inline unsigned blocks_for(std::int64_t n, int per = T) {
      return static_cast<unsigned>((n + per - 1) / per);
    }

    // ------------------------------------------------------------------ device-wide exclusive scan

    constexpr int SCAN_T = 256, SCAN_I = 8, SCAN_B = SCAN_T * SCAN_I;

    __device__ int block_exclusive_sum(int v, int* total) {
      __shared__ int warp_sums[SCAN_T / 32];
      int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      int x = v;
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) warp_sums[warp] = x;
      __syncthreads();
      if (warp == 0) {
        int w = lane < SCAN_T / 32 ? warp_sums[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
          int y = __shfl_up_sync(0xffffffffu, w, o);
          if (lane >= o) w += y;
        }
        if (lane < SCAN_T / 32) warp_sums[lane] = w;
      }
      __syncthreads();
      int const before = warp > 0 ? warp_sums[warp - 1] : 0;
      *total = warp_sums[SCAN_T / 32 - 1];
      __syncthreads();
      return before + x - v;
    }

    __global__ void k_scan_block(int const* in, int* out, std::int64_t n, int* bsum) {
      std::int64_t const base = static_cast<std::int64_t>(blockIdx.x) * SCAN_B + threadIdx.x * SCAN_I;
      int v[SCAN_I];
      int s = 0;
#pragma unroll
      for (int k = 0; k < SCAN_I; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        s += v[k];
      }
      int total;
      int run = block_exclusive_sum(s, &total);
#pragma unroll
      for (int k = 0; k < SCAN_I; ++k) {
        if (base + k < n) out[base + k] = run;
        run += v[k];
      }
      if (threadIdx.x == 0) bsum[blockIdx.x] = total;
    }

    __global__ void k_scan_add(int* out, std::int64_t n, int const* bsum) {
      std::int64_t const base = static_cast<std::int64_t>(blockIdx.x) * SCAN_B + threadIdx.x * SCAN_I;
      int const add = bsum[blockIdx.x];
#pragma unroll
      for (int k = 0; k < SCAN_I; ++k)
        if (base + k < n) out[base + k] += add;
    }

    // ------------------------------------------------------------------ rebuild kernels

    __global__ void k_canon(double const* __restrict__ in, std::int64_t n, GridDesc g, D4* __restrict__ r,
                            int* __restrict__ img, double inv0, double inv1, double inv2) {
      std::int64_t const i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i >= n) return;
      double const x = in[3 * i + 0], y = in[3 * i + 1], z = in[3 * i + 2];
      D4 o;
      o.x = x - g.L[0] * floor(x * inv0);
      o.y = y - g.L[1] * floor(y * inv1);
      o.z = z - g.L[2] * floor(z * inv2);
      o.w = 0;
      r[i] = o;
      img[i] = static_cast<int>(i);
    }

    __device__ inline double comp(D4 const& v, int ax) { return ax == 0 ? v.x : ax == 1 ? v.y : v.z; }

    __global__ void k_ghost_flags(D4 const* __restrict__ r, std::int64_t end, int ax, double rc, double L,
                                  int* __restrict__ fp, int* __restrict__ fm) {
      std::int64_t const j = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (j >= end) return;
      double const x = comp(r[j], ax);
      fp[j] = x < rc ? 1 : 0;
      fm[j] = x > L - rc ? 1 : 0;
    }

    __global__ void k_totals(int const* fp, int const* sp, int const* fm, int const* sm, std::int64_t end, int* out) {
      out[0] = end > 0 ? sp[end - 1] + fp[end - 1] : 0;
      out[1] = end > 0 ? sm[end - 1] + fm[end - 1] : 0;
    }

    __global__ void k_ghost_write(D4* __restrict__ r, int* __restrict__ img, std::int64_t end, int ax, double L,
                                  int const* __restrict__ fp, int const* __restrict__ sp, int const* __restrict__ fm,
                                  int const* __restrict__ sm, int n_plus) {
      std::int64_t const j = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (j >= end) return;
      D4 const v = r[j];
      int const im = img[j];
      if (fp[j]) {
        D4 w = v;
        if (ax == 0) w.x = v.x + L;
        else if (ax == 1) w.y = v.y + L;
        else w.z = v.z + L;
        std::int64_t const s = end + sp[j];
        r[s] = w;
        img[s] = im;
      }
      if (fm[j]) {
        D4 w = v;
        if (ax == 0) w.x = v.x - L;
        else if (ax == 1) w.y = v.y - L;
        else w.z = v.z - L;
        std::int64_t const s = end + n_plus + sm[j];
        r[s] = w;
        img[s] = im;
      }
    }

    __device__ inline int cell_of(D4 const& v, GridDesc const& g) {
      double const c[3] = {v.x, v.y, v.z};
      int idx = 0, stride = 1;
#pragma unroll
      for (int k = 0; k < 3; ++k) {
        int i = static_cast<int>((c[k] + g.cell[k]) * g.inv_cell[k]);
        i = min(max(i, 0), g.shape[k] - 1);
        idx += i * stride;
        stride *= g.shape[k];
      }
      return idx;
    }

    __global__ void k_cell_index(D4 const* __restrict__ r, std::int64_t slots, GridDesc g, int* __restrict__ cell,
                                 int* __restrict__ count) {
      std::int64_t const s = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (s >= slots) return;
      int const c = cell_of(r[s], g);
      cell[s] = c;
      atomicAdd(&count[c], 1);
    }

    __global__ void k_cell_scatter(int const* __restrict__ cell, std::int64_t slots, int const* __restrict__ start,
                                   int* __restrict__ fill, int* __restrict__ members) {
      std::int64_t const s = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (s >= slots) return;
      int const c = cell[s];
      members[start[c] + atomicAdd(&fill[c], 1)] = static_cast<int>(s);
    }

    // Insertion sort of each cell's members into ascending reference slot order (cells hold tens of
    // slots; one thread per cell).
    __global__ void k_cell_sort(int const* __restrict__ start, int const* __restrict__ count, int ncells,
                                int* __restrict__ members) {
      int const c = blockIdx.x * blockDim.x + threadIdx.x;
      if (c >= ncells) return;
      int* m = members + start[c];
      int const k = count[c];
      for (int i = 1; i < k; ++i) {
        int const v = m[i];
        int j = i - 1;
        while (j >= 0 && m[j] > v) {
          m[j + 1] = m[j];
          --j;
        }
        m[j + 1] = v;
      }
    }

    __global__ void k_gather_phys(int const* __restrict__ members, std::int64_t slots, std::int64_t n,
                                  D4 const* __restrict__ r, int const* __restrict__ img, D4* __restrict__ pos,
                                  int* __restrict__ pimg, int* __restrict__ pref, int* __restrict__ real_flag) {
      std::int64_t const p = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (p >= slots) return;
      int const s = members[p];
      pos[p] = r[s];
      pimg[p] = img[s];
      pref[p] = s;
      real_flag[p] = s < n ? 1 : 0;
    }

    __global__ void k_real_compact(int const* __restrict__ flag, int const* __restrict__ scan, std::int64_t slots,
                                   int* __restrict__ real_phys) {
      std::int64_t const p = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (p >= slots) return;
      if (flag[p]) real_phys[scan[p]] = static_cast<int>(p);
    }

    // Binary32 hi parts of the offset coordinates of every physical slot (for the build prefilter).
    __global__ void k_hi(D4 const* __restrict__ pos, std::int64_t slots, float4* __restrict__ hi, double sx, double sy,
                         double sz) {
      std::int64_t const p = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (p >= slots) return;
      D4 const v = pos[p];
      hi[p] = make_float4(static_cast<float>(v.x + sx), static_cast<float>(v.y + sy), static_cast<float>(v.z + sz), 0.f);
    }

    // Per real atom j (cell order): own cell (skipping itself) then the adjacent cells in increasing
    // index, each walked from its last physical slot down. Records physical neighbour slots.
    // The binary32 hi coordinates lie in one binade per axis, so their differences are exact and the
    // binary32 r^2 is within `band` of the binary64 one; only candidates inside that band take the
    // binary64 test (dx*dx + dy*dy) + dz*dz < rc^2, which is the decision the reference makes.
    __global__ void k_build(D4 const* __restrict__ pos, float4 const* __restrict__ hi, int const* __restrict__ real_phys,
                            int const* __restrict__ cell_ref, int const* __restrict__ pref,
                            int const* __restrict__ start, int const* __restrict__ count, std::int64_t n, GridDesc g,
                            float band, int cap, int* __restrict__ nbr, int* __restrict__ ncount,
                            int* __restrict__ maxc) {
      std::int64_t const j = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (j >= n) return;
      int const p = real_phys[j];
      float4 const hp = hi[p];
      double const rc2 = g.rc * g.rc;
      float const lo_f = static_cast<float>(rc2) - band, hi_f = static_cast<float>(rc2) + band;
      int const c = cell_ref[pref[p]];
      int const s0 = g.shape[0], s1 = g.shape[1], s2 = g.shape[2];
      int const cx = c % s0, cy = (c / s0) % s1, cz = c / (s0 * s1);
      int k = 0;
      auto scan = [&](int cell, bool same) {
        int const b = start[cell];
        for (int q = b + count[cell] - 1; q >= b; --q) {
          if (same && q == p) continue;
          float4 const hq = hi[q];
          float const fx = hp.x - hq.x, fy = hp.y - hq.y, fz = hp.z - hq.z;
          float const r2f = fx * fx + fy * fy + fz * fz;
          bool in = r2f < lo_f;
          if (!in && r2f <= hi_f) {
            D4 const ri = pos[p], rq = pos[q];
            double const dx = ri.x - rq.x, dy = ri.y - rq.y, dz = ri.z - rq.z;
            in = (dx * dx + dy * dy) + dz * dz < rc2;
          }
          if (in) {
            if (k < cap) nbr[static_cast<std::int64_t>(k) * n + j] = q;
            ++k;
          }
        }
      };
      scan(c, true);
      for (int z = max(cz - 1, 0); z < min(cz + 2, s2); ++z)
        for (int y = max(cy - 1, 0); y < min(cy + 2, s1); ++y)
          for (int x = max(cx - 1, 0); x < min(cx + 2, s0); ++x) {
            int const m = x + y * s0 + z * s0 * s1;
            if (m != c) scan(m, false);
          }
      ncount[j] = k;
      if (k > cap) atomicMax(maxc, k);
    }

    __global__ void k_update(D4* __restrict__ pos, int const* __restrict__ pimg, std::int64_t slots,
                             double const* __restrict__ d, Packed* __restrict__ packed, double sx, double sy,
                             double sz) {
      std::int64_t const p = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (p >= slots) return;
      std::int64_t const i = pimg[p];
      D4 v = pos[p];
      v.x = v.x - d[3 * i + 0];
      v.y = v.y - d[3 * i + 1];
      v.z = v.z - d[3 * i + 2];
      pos[p] = v;
      if (packed) {
        double const X = v.x + sx, Y = v.y + sy, Z = v.z + sz;
        float const hx = static_cast<float>(X), hy = static_cast<float>(Y), hz = static_cast<float>(Z);
        Packed& q = packed[p];
        q.hx = hx;
        q.hy = hy;
        q.hz = hz;
        q.lx = static_cast<float>(X - static_cast<double>(hx));
        q.ly = static_cast<float>(Y - static_cast<double>(hy));
        q.lz = static_cast<float>(Z - static_cast<double>(hz));
      }
    }

    __global__ void k_pack(D4 const* __restrict__ pos, int const* __restrict__ ptype, std::int64_t slots,
                           Packed* __restrict__ packed, double sx, double sy, double sz) {
      std::int64_t const p = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (p >= slots) return;
      D4 const v = pos[p];
      double const X = v.x + sx, Y = v.y + sy, Z = v.z + sz;
      float const hx = static_cast<float>(X), hy = static_cast<float>(Y), hz = static_cast<float>(Z);
      Packed q;
      q.hx = hx;
      q.hy = hy;
      q.hz = hz;
      q.type = static_cast<std::uint32_t>(ptype[p]);
      q.lx = static_cast<float>(X - static_cast<double>(hx));
      q.ly = static_cast<float>(Y - static_cast<double>(hy));
      q.lz = static_cast<float>(Z - static_cast<double>(hz));
      q.fp = 0.f;
      packed[p] = q;
    }

    __global__ void k_types_phys(int const* __restrict__ pimg, std::int64_t slots, std::uint32_t const* __restrict__ types,
                                 int n_types_guard, int* __restrict__ ptype, int* __restrict__ err) {
      std::int64_t const p = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (p >= slots) return;
      std::uint32_t t = types[pimg[p]];
      if (n_types_guard > 0 && t >= static_cast<std::uint32_t>(n_types_guard)) {
        atomicOr(err, ERR_BAD_INDEX);
        t = 0;
      }
      ptype[p] = static_cast<int>(t);
    }

    // Neighbours within r_cut of real atom j, in list order (export for parity checks).
    __global__ void k_export_count(D4 const* __restrict__ pos, int const* __restrict__ real_phys,
                                   int const* __restrict__ pimg, int const* __restrict__ nbr,
                                   int const* __restrict__ ncount, std::int64_t n, double rc2,
                                   int* __restrict__ counts) {
      std::int64_t const j = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (j >= n) return;
      int const p = real_phys[j];
      D4 const ri = pos[p];
      int c = 0;
      int const nc = ncount[j];
      int k = 0;
      // four neighbours' loads in flight together
      for (; k + 4 <= nc; k += 4) {
        D4 rq[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) rq[u] = pos[nbr[static_cast<std::int64_t>(k + u) * n + j]];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          double const dx = rq[u].x - ri.x, dy = rq[u].y - ri.y, dz = rq[u].z - ri.z;
          if ((dx * dx + dy * dy) + dz * dz < rc2) ++c;
        }
      }
      for (; k < nc; ++k) {
        D4 const rq = pos[nbr[static_cast<std::int64_t>(k) * n + j]];
        double const dx = rq.x - ri.x, dy = rq.y - ri.y, dz = rq.z - ri.z;
        if ((dx * dx + dy * dy) + dz * dz < rc2) ++c;
      }
      counts[pimg[p]] = c;
    }

    // The neighbours within r_cut of one real atom, in list order: real indices and r_n - r_i.
    __global__ void k_export_one(D4 const* __restrict__ pos, int const* __restrict__ real_phys,
                                 int const* __restrict__ pimg, int const* __restrict__ nbr,
                                 int const* __restrict__ ncount, std::int64_t n, double rc2, std::int64_t atom, int cap,
                                 int* __restrict__ idx, double* __restrict__ dr, int* __restrict__ count) {
      std::int64_t const j = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (j >= n) return;
      int const p = real_phys[j];
      if (pimg[p] != atom) return;
      D4 const ri = pos[p];
      int c = 0;
      for (int k = 0; k < ncount[j]; ++k) {
        int const q = nbr[static_cast<std::int64_t>(k) * n + j];
        D4 const rq = pos[q];
        double const dx = rq.x - ri.x, dy = rq.y - ri.y, dz = rq.z - ri.z;
        if ((dx * dx + dy * dy) + dz * dz < rc2) {
          if (c < cap) {
            idx[c] = pimg[q];
            dr[3 * c + 0] = dx;
            dr[3 * c + 1] = dy;
            dr[3 * c + 2] = dz;
          }
          ++c;
        }
      }
      *count = c;
    }

    __global__ void k_export_fill(D4 const* __restrict__ pos, int const* __restrict__ real_phys,
                                  int const* __restrict__ pimg, int const* __restrict__ nbr,
                                  int const* __restrict__ ncount, std::int64_t n, double rc2,
                                  long long const* __restrict__ offs, int* __restrict__ idx, double* __restrict__ dr) {
      std::int64_t const j = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (j >= n) return;
      int const p = real_phys[j];
      D4 const ri = pos[p];
      long long o = offs[pimg[p]];
      int const nc = ncount[j];
      int k = 0;
      // four neighbours' loads in flight together, written in list order
      for (; k + 4 <= nc; k += 4) {
        int q[4], im[4];
        D4 rq[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) q[u] = nbr[static_cast<std::int64_t>(k + u) * n + j];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          rq[u] = pos[q[u]];
          im[u] = pimg[q[u]];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          double const dx = rq[u].x - ri.x, dy = rq[u].y - ri.y, dz = rq[u].z - ri.z;
          if ((dx * dx + dy * dy) + dz * dz < rc2) {
            idx[o] = im[u];
            dr[3 * o + 0] = dx;
            dr[3 * o + 1] = dy;
            dr[3 * o + 2] = dz;
            ++o;
          }
        }
      }
      for (; k < nc; ++k) {
        int const q = nbr[static_cast<std::int64_t>(k) * n + j];
        D4 const rq = pos[q];
        double const dx = rq.x - ri.x, dy = rq.y - ri.y, dz = rq.z - ri.z;
        if ((dx * dx + dy * dy) + dz * dz < rc2) {
          idx[o] = pimg[q];
          dr[3 * o + 0] = dx;
          dr[3 * o + 1] = dy;
          dr[3 * o + 2] = dz;
          ++o;
        }
      }
    }

    void sync_small(flygpu_list* L, int count) {
      FLY_CUDA(cudaMemcpyAsync(L->h_small.p, L->counters.p, sizeof(int) * count, cudaMemcpyDeviceToHost, L->stream));
      FLY_CUDA(cudaStreamSynchronize(L->stream));
    }

  }  // namespace

  std::size_t scan_tmp_size(std::int64_t n) {
    std::size_t total = 64;
    while (n > 1) {
      n = (n + SCAN_B - 1) / SCAN_B;
      total += static_cast<std::size_t>(n) + 1;
    }
    return total;
  }

  void exclusive_scan(int const* in, int* out, std::int64_t n, int* tmp, std::size_t tmp_len, cudaStream_t s) {
    if (n <= 0) return;
    std::int64_t const nb = (n + SCAN_B - 1) / SCAN_B;
    if (static_cast<std::size_t>(nb) > tmp_len) fail(FLYGPU_CUDA_ERROR, "scan scratch too small");
    launch(k_scan_block, static_cast<unsigned>(nb), SCAN_T, 0, s, in, out, n, tmp);
    if (nb > 1) {
      exclusive_scan(tmp, tmp, nb, tmp + nb, tmp_len - static_cast<std::size_t>(nb), s);
      launch(k_scan_add, static_cast<unsigned>(nb), SCAN_T, 0, s, out, n, tmp);
    }
    FLY_CUDA(cudaGetLastError());
  }

  void list_rebuild(flygpu_list* L, double const* d_pos, std::int64_t n) {
    if (n < 0) fail(FLYGPU_INVALID_ARG, "negative atom count");
    if (n * 27 >= (std::int64_t{1} << 31)) fail(FLYGPU_INVALID_ARG, "too many atoms for 32-bit slot indices");
    cudaStream_t const s = L->stream;
    GridDesc const& g = L->g;
    if (n != L->n) {
      L->n = n;
      L->types_set = false;
      L->frozen_set = false;
      L->nb_cap = 0;
    }
    L->n_slots = 0;
    L->built = false;
    L->packed_valid = false;
    L->counters.reserve(8);
    L->h_small.reserve(8);
    L->err.reserve(1);
    if (n == 0) {
      L->built = true;
      return;
    }
    cudaEvent_t const t_start = timer_record(L);
    std::int64_t const cap_slots = n * 27;  // real + MAX_GHOST_RATIO * n (neigh/list.hpp:78)
    std::size_t guess = static_cast<std::size_t>(n + n / 2 + 1024);
    L->r_ref.reserve(guess);
    L->img_ref.reserve(guess);
    launch(k_canon, blocks_for(n), T, 0, s, d_pos, n, g, L->r_ref.p, L->img_ref.p, 1.0 / g.L[0], 1.0 / g.L[1], 1.0 / g.L[2]);
    FLY_CUDA(cudaGetLastError());
    std::int64_t slots = n;
    for (int ax = 0; ax < 3; ++ax) {
      if (!g.per[ax]) continue;
      std::int64_t const end = slots;
      L->flag_p.reserve(static_cast<std::size_t>(end));
      L->flag_m.reserve(static_cast<std::size_t>(end));
      L->scan_p.reserve(static_cast<std::size_t>(end));
      L->scan_m.reserve(static_cast<std::size_t>(end));
      L->scan_tmp.reserve(scan_tmp_size(end));
      launch(k_ghost_flags, blocks_for(end), T, 0, s, L->r_ref.p, end, ax, g.rc, g.L[ax], L->flag_p.p, L->flag_m.p);
      exclusive_scan(L->flag_p.p, L->scan_p.p, end, L->scan_tmp.p, L->scan_tmp.n, s);
      exclusive_scan(L->flag_m.p, L->scan_m.p, end, L->scan_tmp.p, L->scan_tmp.n, s);
      launch(k_totals, 1, 1, 0, s, L->flag_p.p, L->scan_p.p, L->flag_m.p, L->scan_m.p, end, L->counters.p);
      FLY_CUDA(cudaGetLastError());
      sync_small(L, 2);
      std::int64_t const tp = L->h_small.p[0], tm = L->h_small.p[1];
      std::int64_t const next = end + tp + tm;
      if (next > cap_slots)
        fail(FLYGPU_GHOST_OVERFLOW, "more than MAX_GHOST_RATIO * n ghost atoms");
      L->r_ref.grow_keep(static_cast<std::size_t>(next), static_cast<std::size_t>(end), s);
      L->img_ref.grow_keep(static_cast<std::size_t>(next), static_cast<std::size_t>(end), s);
      launch(k_ghost_write, blocks_for(end), T, 0, s, L->r_ref.p, L->img_ref.p, end, ax, g.L[ax], L->flag_p.p, L->scan_p.p,
                                                  L->flag_m.p, L->scan_m.p, static_cast<int>(tp));
      FLY_CUDA(cudaGetLastError());
      slots = next;
    }
    L->n_slots = slots;
    int const nc = g.ncells();
    L->cell_count.reserve(static_cast<std::size_t>(nc));
    L->cell_start.reserve(static_cast<std::size_t>(nc));
    L->cell_fill.reserve(static_cast<std::size_t>(nc));
    L->cell_ref.reserve(static_cast<std::size_t>(slots));
    L->members.reserve(static_cast<std::size_t>(slots));
    L->scan_tmp.reserve(scan_tmp_size(std::max<std::int64_t>(nc, slots)));
    FLY_CUDA(cudaMemsetAsync(L->cell_count.p, 0, sizeof(int) * static_cast<std::size_t>(nc), s));
    FLY_CUDA(cudaMemsetAsync(L->cell_fill.p, 0, sizeof(int) * static_cast<std::size_t>(nc), s));
    launch(k_cell_index, blocks_for(slots), T, 0, s, L->r_ref.p, slots, g, L->cell_ref.p, L->cell_count.p);
    exclusive_scan(L->cell_count.p, L->cell_start.p, nc, L->scan_tmp.p, L->scan_tmp.n, s);
    launch(k_cell_scatter, blocks_for(slots), T, 0, s, L->cell_ref.p, slots, L->cell_start.p, L->cell_fill.p, L->members.p);
    launch(k_cell_sort, blocks_for(nc, 128), 128, 0, s, L->cell_start.p, L->cell_count.p, nc, L->members.p);
    FLY_CUDA(cudaGetLastError());
    L->pos.reserve(static_cast<std::size_t>(slots));
    L->pimg.reserve(static_cast<std::size_t>(slots));
    L->pref.reserve(static_cast<std::size_t>(slots));
    L->ptype.reserve(static_cast<std::size_t>(slots));
    L->flag_p.reserve(static_cast<std::size_t>(slots));
    L->scan_p.reserve(static_cast<std::size_t>(slots));
    L->real_phys.reserve(static_cast<std::size_t>(n));
    launch(k_gather_phys, blocks_for(slots), T, 0, s, L->members.p, slots, n, L->r_ref.p, L->img_ref.p, L->pos.p, L->pimg.p,
                                                   L->pref.p, L->flag_p.p);
    exclusive_scan(L->flag_p.p, L->scan_p.p, slots, L->scan_tmp.p, L->scan_tmp.n, s);
    launch(k_real_compact, blocks_for(slots), T, 0, s, L->flag_p.p, L->scan_p.p, slots, L->real_phys.p);
    FLY_CUDA(cudaGetLastError());
    // Neighbour lists; grow the capacity once if any atom overflowed it. The first capacity is the
    // expected count at the real-atom density plus headroom.
    L->ncount.reserve(static_cast<std::size_t>(n));
    L->hi.reserve(static_cast<std::size_t>(slots));
    launch(k_hi, blocks_for(slots), T, 0, s, L->pos.p, slots, L->hi.p, L->shift[0], L->shift[1], L->shift[2]);
    if (L->nb_cap == 0) {
      double const vol = g.L[0] * g.L[1] * g.L[2];
      double const expect = 4.18879 * g.rc * g.rc * g.rc * static_cast<double>(n) / vol;
      L->nb_cap = std::min(1024, (static_cast<int>(1.25 * expect) + 16 + 7) / 8 * 8);
    }
    // Error bound of the binary32 r^2 (hi parts carry at most half an ulp of the offset binade each).
    double ulp = 0;
    for (int k = 0; k < 3; ++k) ulp = std::max(ulp, std::ldexp(1.0, std::ilogb(L->shift[k] + g.L[k]) - 23));
    float const band = static_cast<float>(4.0 * g.rc * std::sqrt(3.0) * ulp + 1e-5 * g.rc * g.rc + 1e-6);
    for (int attempt = 0; attempt < 2; ++attempt) {
      L->nbr.reserve(static_cast<std::size_t>(L->nb_cap) * static_cast<std::size_t>(n));
      FLY_CUDA(cudaMemsetAsync(L->counters.p + 2, 0, sizeof(int), s));
      launch(k_build, blocks_for(n, 128), 128, 0, s, L->pos.p, L->hi.p, L->real_phys.p, L->cell_ref.p, L->pref.p,
             L->cell_start.p, L->cell_count.p, n, g, band, L->nb_cap, L->nbr.p, L->ncount.p, L->counters.p + 2);
      FLY_CUDA(cudaGetLastError());
      sync_small(L, 3);
      int const need = L->h_small.p[2];
      if (need <= L->nb_cap) break;
      if (attempt == 1) fail(FLYGPU_NLIST_OVERFLOW, "neighbour capacity exceeded");
      L->nb_cap = (need + 7) / 8 * 8;
    }
    if (L->types_set) {
      launch(k_types_phys, blocks_for(slots), T, 0, s, L->pimg.p, slots, L->types.p, 0, L->ptype.p, L->err.p);
      FLY_CUDA(cudaGetLastError());
    }
    timer_mark(L, TK_REBUILD, t_start, timer_record(L));
    L->built = true;
  }

  void list_update(flygpu_list* L, double const* d_delta) {
    if (!L->built) fail(FLYGPU_INVALID_ARG, "update() before rebuild()");
    if (L->n_slots == 0) return;
    Packed* pk = L->packed_valid ? L->packed.p : nullptr;
    cudaEvent_t const t0 = timer_record(L);
    launch(k_update, blocks_for(L->n_slots), T, 0, L->stream, L->pos.p, L->pimg.p, L->n_slots, d_delta, pk, L->shift[0],
                                                           L->shift[1], L->shift[2]);
    timer_mark(L, TK_UPDATE, t0, timer_record(L));
    FLY_CUDA(cudaGetLastError());
  }

  void list_set_atoms(flygpu_list* L, int n_types, std::uint32_t const* d_types, std::uint8_t const* d_frozen,
                      bool from_host, std::uint32_t const* h_types, std::uint8_t const* h_frozen) {
    if (!L->built) fail(FLYGPU_INVALID_ARG, "EAM call before List::rebuild()");
    std::size_t const n = static_cast<std::size_t>(L->n);
    L->types.reserve(n + 1);
    L->frozen.reserve(n + 1);
    bool types_changed = false;
    if (from_host) {
      if (h_types) {
        for (std::size_t i = 0; i < n; ++i)
          if (h_types[i] >= static_cast<std::uint32_t>(n_types)) fail(FLYGPU_INVALID_ARG, "type index out of range");
        FLY_CUDA(cudaMemcpyAsync(L->types.p, h_types, n * sizeof(std::uint32_t), cudaMemcpyHostToDevice, L->stream));
        types_changed = true;
      }
      if (h_frozen) FLY_CUDA(cudaMemcpyAsync(L->frozen.p, h_frozen, n, cudaMemcpyHostToDevice, L->stream));
    } else {
      if (d_types) {
        FLY_CUDA(cudaMemcpyAsync(L->types.p, d_types, n * sizeof(std::uint32_t), cudaMemcpyDeviceToDevice, L->stream));
        types_changed = true;
      }
      if (d_frozen) FLY_CUDA(cudaMemcpyAsync(L->frozen.p, d_frozen, n, cudaMemcpyDeviceToDevice, L->stream));
    }
    if (!types_changed && !L->types_set) fail(FLYGPU_INVALID_ARG, "types were never provided");
    if ((from_host ? h_frozen : d_frozen) != nullptr) {
      L->frozen_set = true;
    } else if (!L->frozen_set) {
      FLY_CUDA(cudaMemsetAsync(L->frozen.p, 0, n, L->stream));  // no frozen flags given: all atoms active
      L->frozen_set = true;
    }
    if (types_changed && L->n_slots > 0) {
      launch(k_types_phys, blocks_for(L->n_slots), T, 0, L->stream, L->pimg.p, L->n_slots, L->types.p, n_types,
                                                                L->ptype.p, L->err.p);
      FLY_CUDA(cudaGetLastError());
      L->packed_valid = false;
    }
    if (types_changed) L->types_set = true;
  }

  void list_pack(flygpu_list* L) {
    if (L->packed_valid || L->n_slots == 0) return;
    L->packed.reserve(static_cast<std::size_t>(L->n_slots));
    launch(k_pack, blocks_for(L->n_slots), T, 0, L->stream, L->pos.p, L->ptype.p, L->n_slots, L->packed.p, L->shift[0],
                                                         L->shift[1], L->shift[2]);
    FLY_CUDA(cudaGetLastError());
    L->packed_valid = true;
  }

  int list_take_error(flygpu_list* L) {
    L->err.reserve(1);
    L->h_small.reserve(8);
    FLY_CUDA(cudaMemcpyAsync(L->h_small.p + 4, L->err.p, sizeof(int), cudaMemcpyDeviceToHost, L->stream));
    FLY_CUDA(cudaStreamSynchronize(L->stream));
    int const w = L->h_small.p[4];
    if (w) FLY_CUDA(cudaMemsetAsync(L->err.p, 0, sizeof(int), L->stream));
    return w;
  }

  std::int64_t list_export(flygpu_list* L, double r_cut, int* counts, int* idx, double* dr, std::int64_t cap) {
    if (!L->built) fail(FLYGPU_INVALID_ARG, "neighbours() before rebuild()");
    if (r_cut > L->g.rc) fail(FLYGPU_INVALID_ARG, "r_cut is bigger than the list's cut-off");
    std::int64_t const n = L->n;
    if (n == 0) return 0;
    cudaStream_t const s = L->stream;
    double const rc2 = r_cut * r_cut;
    DevBuf<int> d_counts, d_idx;
    DevBuf<long long> d_offs;
    DevBuf<double> d_dr;
    d_counts.reserve(static_cast<std::size_t>(n));
    launch(k_export_count, blocks_for(n), T, 0, s, L->pos.p, L->real_phys.p, L->pimg.p, L->nbr.p, L->ncount.p, n, rc2,
                                               d_counts.p);
    FLY_CUDA(cudaGetLastError());
    std::vector<int> hc(static_cast<std::size_t>(n));
    FLY_CUDA(cudaMemcpyAsync(hc.data(), d_counts.p, sizeof(int) * hc.size(), cudaMemcpyDeviceToHost, s));
    FLY_CUDA(cudaStreamSynchronize(s));
    std::vector<long long> offs(static_cast<std::size_t>(n));
    long long total = 0;
    for (std::int64_t i = 0; i < n; ++i) {
      offs[static_cast<std::size_t>(i)] = total;
      total += hc[static_cast<std::size_t>(i)];
    }
    if (counts) std::copy(hc.begin(), hc.end(), counts);
    if (idx && dr && cap >= total && total > 0) {
      d_offs.reserve(static_cast<std::size_t>(n));
      d_idx.reserve(static_cast<std::size_t>(total));
      d_dr.reserve(static_cast<std::size_t>(3 * total));
      FLY_CUDA(cudaMemcpyAsync(d_offs.p, offs.data(), sizeof(long long) * offs.size(), cudaMemcpyHostToDevice, s));
      launch(k_export_fill, blocks_for(n), T, 0, s, L->pos.p, L->real_phys.p, L->pimg.p, L->nbr.p, L->ncount.p, n, rc2,
                                                d_offs.p, d_idx.p, d_dr.p);
      FLY_CUDA(cudaGetLastError());
      FLY_CUDA(cudaMemcpyAsync(idx, d_idx.p, sizeof(int) * static_cast<std::size_t>(total), cudaMemcpyDeviceToHost, s));
      FLY_CUDA(cudaMemcpyAsync(dr, d_dr.p, sizeof(double) * static_cast<std::size_t>(3 * total), cudaMemcpyDeviceToHost, s));
      FLY_CUDA(cudaStreamSynchronize(s));
    }
    return total;
  }

  int list_neighbours_of(flygpu_list* L, double r_cut, std::int64_t atom, std::vector<int>& idx,
                         std::vector<double>& dr) {
    if (!L->built) fail(FLYGPU_INVALID_ARG, "neighbours() before rebuild()");
    if (r_cut > L->g.rc) fail(FLYGPU_INVALID_ARG, "r_cut is bigger than the list's cut-off");
    if (atom < 0 || atom >= L->n) fail(FLYGPU_INVALID_ARG, "atom index out of range");
    cudaStream_t const s = L->stream;
    int const cap = std::max(1, L->nb_cap);
    DevBuf<int> d_idx, d_cnt;
    DevBuf<double> d_dr;
    d_idx.reserve(static_cast<std::size_t>(cap));
    d_cnt.reserve(1);
    d_dr.reserve(3 * static_cast<std::size_t>(cap));
    launch(k_export_one, blocks_for(L->n), T, 0, s, L->pos.p, L->real_phys.p, L->pimg.p, L->nbr.p, L->ncount.p, L->n,
           r_cut * r_cut, atom, cap, d_idx.p, d_dr.p, d_cnt.p);
    int c = 0;
    FLY_CUDA(cudaMemcpyAsync(&c, d_cnt.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    FLY_CUDA(cudaStreamSynchronize(s));
    c = std::min(c, cap);
    idx.resize(static_cast<std::size_t>(c));
    dr.resize(3 * static_cast<std::size_t>(c));
    if (c > 0) {
      FLY_CUDA(cudaMemcpyAsync(idx.data(), d_idx.p, sizeof(int) * idx.size(), cudaMemcpyDeviceToHost, s));
      FLY_CUDA(cudaMemcpyAsync(dr.data(), d_dr.p, sizeof(double) * dr.size(), cudaMemcpyDeviceToHost, s));
      FLY_CUDA(cudaStreamSynchronize(s));
    }
    return c;
  }

  std::vector<int> list_export_device(flygpu_list* L, double r_cut, DevBuf<long long>& offs, DevBuf<int>& idx,
                                      DevBuf<double>& dr) {
    if (!L->built) fail(FLYGPU_INVALID_ARG, "neighbours() before rebuild()");
    if (r_cut > L->g.rc) fail(FLYGPU_INVALID_ARG, "r_cut is bigger than the list's cut-off");
    std::int64_t const n = L->n;
    std::vector<int> hc(static_cast<std::size_t>(n));
    if (n == 0) return hc;
    cudaStream_t const s = L->stream;
    double const rc2 = r_cut * r_cut;
    DevBuf<int>& d_counts = L->export_counts;
    d_counts.reserve(static_cast<std::size_t>(n));
    launch(k_export_count, blocks_for(n), T, 0, s, L->pos.p, L->real_phys.p, L->pimg.p, L->nbr.p, L->ncount.p, n, rc2,
           d_counts.p);
    FLY_CUDA(cudaMemcpyAsync(hc.data(), d_counts.p, sizeof(int) * hc.size(), cudaMemcpyDeviceToHost, s));
    FLY_CUDA(cudaStreamSynchronize(s));
    std::vector<long long> ho(static_cast<std::size_t>(n) + 1);
    long long total = 0;
    for (std::int64_t i = 0; i < n; ++i) {
      ho[static_cast<std::size_t>(i)] = total;
      total += hc[static_cast<std::size_t>(i)];
    }
    ho[static_cast<std::size_t>(n)] = total;
    offs.reserve(static_cast<std::size_t>(n) + 1);
    idx.reserve(static_cast<std::size_t>(std::max<long long>(total, 1)));
    dr.reserve(static_cast<std::size_t>(3 * std::max<long long>(total, 1)));
    // a copy from pageable memory returns once the driver has staged it, so ho may go out of scope
    FLY_CUDA(cudaMemcpyAsync(offs.p, ho.data(), sizeof(long long) * ho.size(), cudaMemcpyHostToDevice, s));
    if (total > 0)
      launch(k_export_fill, blocks_for(n), T, 0, s, L->pos.p, L->real_phys.p, L->pimg.p, L->nbr.p, L->ncount.p, n, rc2,
             offs.p, idx.p, dr.p);
    return hc;
  }

}  // namespace flygpu
