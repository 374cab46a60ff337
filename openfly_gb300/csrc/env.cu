// env.cu -- the catalogue's local environments of every atom, from the device neighbour list.
//
// Restates, per atom i (binary64, in the reference's operation order; compiled with -fmad=false):
//   env/geometry.hpp:391-407  rebuild_geo_from_nl: the atom itself at (0,0,0), then its neighbours
//                             within r_env in the list's order (for_neighbours, neigh/list.hpp:139-154),
//                             colour 2 type + frozen (to_colour, geometry.hpp:383-385), then the origin
//                             moved to the centroid (Geometry::centre, geometry.hpp:298-305; centroid:
//                             a sequential sum divided by the count, utility/lattice.hpp:203-209);
//   env/heuristics.hpp:93-110 Fingerprint::rebuild: r_0j = |q_j - q_0| (j >= 1) and r_ij = |q_i - q_j|
//                             (1 <= j < i), each sorted ascending; |d| = sqrt((dx^2 + dy^2) + dz^2)
//                             (gnorm, utility/core.hpp:634-680).
// The graph hash that follows (canon_hash, nauty) stays on the host.
//
// Layout: atom i owns geometry entries [geo_off[i], geo_off[i+1]) (geo_off[i] = offs[i] + i), r_0j values
// [geo_off[i] - i, geo_off[i+1] - i - 1) and r_ij values [rij_off[i], rij_off[i+1]). Each atom's two
// distance lists are sorted by one CTA in shared memory (bitonic, padded with +inf).

#include <cmath>
#include <memory>
#include <vector>

#include "internal.hpp"

struct flygpu_env {
  std::int64_t n = 0, n_geo = 0, n_rij = 0;
  std::vector<std::int64_t> geo_off, rij_off;  // n + 1 each (host)
  flygpu::DevBuf<double> pos, r0j, rij;
  flygpu::DevBuf<int> colour, index;
};

namespace flygpu {

  namespace {

    constexpr int SORT_CAP = 8192;  // values of one sorted list that one CTA holds (64 KB)

    __global__ void k_env_geo(std::int64_t n, long long const* __restrict__ offs, int const* __restrict__ idx,
                              double const* __restrict__ dr, std::uint32_t const* __restrict__ types,
                              std::uint8_t const* __restrict__ frozen, double* __restrict__ pos,
                              int* __restrict__ colour, int* __restrict__ index) {
      std::int64_t const i = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (i >= n) return;
      long long const o = offs[i];
      long long const cnt = offs[i + 1] - o;  // offs has n + 1 entries
      std::int64_t const go = o + i;
      double sx = 0.0, sy = 0.0, sz = 0.0;  // centroid: Vec::Zero() += each position in order, the atom's own
      sx += 0.0;                            // (0, 0, 0) first
      sy += 0.0;
      sz += 0.0;
      for (long long k = 0; k < cnt; ++k) {
        sx += dr[3 * (o + k) + 0];
        sy += dr[3 * (o + k) + 1];
        sz += dr[3 * (o + k) + 2];
      }
      double const K = static_cast<double>(cnt + 1);
      double const cx = sx / K, cy = sy / K, cz = sz / K;
      pos[3 * go + 0] = 0.0 - cx;
      pos[3 * go + 1] = 0.0 - cy;
      pos[3 * go + 2] = 0.0 - cz;
      colour[go] = static_cast<int>(2 * types[i] + frozen[i]);
      index[go] = static_cast<int>(i);
      for (long long k = 0; k < cnt; ++k) {
        std::int64_t const g = go + 1 + k;
        pos[3 * g + 0] = dr[3 * (o + k) + 0] - cx;
        pos[3 * g + 1] = dr[3 * (o + k) + 1] - cy;
        pos[3 * g + 2] = dr[3 * (o + k) + 2] - cz;
        int const q = idx[o + k];
        colour[g] = static_cast<int>(2 * types[q] + frozen[q]);
        index[g] = q;
      }
    }

    __device__ inline double norm3(double x, double y, double z) { return sqrt((x * x + y * y) + z * z); }

    // Ascending bitonic sort of v[0, m) (m a power of two) by the whole block.
    __device__ void bitonic(double* v, int m) {
      for (int k = 2; k <= m; k <<= 1) {
        for (int j = k >> 1; j > 0; j >>= 1) {
          for (int t = threadIdx.x; t < m; t += blockDim.x) {
            int const u = t ^ j;
            if (u > t) {
              bool const up = (t & k) == 0;
              double const a = v[t], b = v[u];
              if ((a > b) == up) {
                v[t] = b;
                v[u] = a;
              }
            }
          }
          __syncthreads();
        }
      }
    }

    // One CTA per atom: its r_0j and r_ij lists, each sorted ascending.
    __global__ void k_env_fp(std::int64_t n, long long const* __restrict__ geo_off, long long const* __restrict__ rij_off,
                             double const* __restrict__ pos, double* __restrict__ r0j, double* __restrict__ rij) {
      extern __shared__ double v[];
      std::int64_t const i = blockIdx.x;
      if (i >= n) return;
      long long const go = geo_off[i];
      int const K = static_cast<int>(geo_off[i + 1] - go);
      double const* q = pos + 3 * go;
      // r_0j
      int const m0 = K - 1;
      int p0 = 1;
      while (p0 < m0) p0 <<= 1;
      for (int t = threadIdx.x; t < p0; t += blockDim.x) {
        v[t] = t < m0 ? norm3(q[3 * (t + 1) + 0] - q[0], q[3 * (t + 1) + 1] - q[1], q[3 * (t + 1) + 2] - q[2])
                      : INFINITY;
      }
      __syncthreads();
      bitonic(v, p0);
      for (int t = threadIdx.x; t < m0; t += blockDim.x) r0j[go - i + t] = v[t];
      __syncthreads();
      // r_ij, 1 <= j < a < K: pair t -> (a, j) with a(a-1)/2 - ... enumerated row by row
      long long const ro = rij_off[i];
      int const m1 = static_cast<int>(rij_off[i + 1] - ro);
      int p1 = 1;
      while (p1 < m1) p1 <<= 1;
      for (int t = threadIdx.x; t < p1; t += blockDim.x) {
        double r = INFINITY;
        if (t < m1) {
          // row a (>= 2) holds pairs (a, 1..a-1): rows start at (a-1)(a-2)/2
          int a = static_cast<int>(floor((1.0 + sqrt(1.0 + 8.0 * static_cast<double>(t))) * 0.5)) + 1;
          while ((a - 1) * (a - 2) / 2 > t) --a;
          while (a * (a - 1) / 2 <= t) ++a;
          int const j = t - (a - 1) * (a - 2) / 2 + 1;
          r = norm3(q[3 * a + 0] - q[3 * j + 0], q[3 * a + 1] - q[3 * j + 1], q[3 * a + 2] - q[3 * j + 2]);
        }
        v[t] = r;
      }
      __syncthreads();
      bitonic(v, p1);
      for (int t = threadIdx.x; t < m1; t += blockDim.x) rij[ro + t] = v[t];
    }

  }  // namespace

  flygpu_env* env_build(flygpu_list* L, double r_env, std::uint32_t const* h_types, std::uint8_t const* h_frozen) {
    if (!(r_env > 0)) fail(FLYGPU_INVALID_ARG, "r_env must be positive");
    auto E = std::make_unique<flygpu_env>();
    DevBuf<long long> offs;
    DevBuf<int> idx;
    DevBuf<double> dr;
    std::vector<int> const cnt = list_export_device(L, r_env, offs, idx, dr);
    std::int64_t const n = L->n;
    E->n = n;
    E->geo_off.assign(static_cast<std::size_t>(n) + 1, 0);
    E->rij_off.assign(static_cast<std::size_t>(n) + 1, 0);
    std::int64_t nb = 0;
    for (std::int64_t i = 0; i < n; ++i) {
      std::int64_t const c = cnt[static_cast<std::size_t>(i)];
      if (c + 1 > SORT_CAP || c * (c - 1) / 2 > SORT_CAP)
        fail(FLYGPU_INVALID_ARG, "local environment too large to sort on the device (r_env too big)");
      E->geo_off[static_cast<std::size_t>(i) + 1] = E->geo_off[static_cast<std::size_t>(i)] + c + 1;
      E->rij_off[static_cast<std::size_t>(i) + 1] = E->rij_off[static_cast<std::size_t>(i)] + c * (c - 1) / 2;
      nb += c;
    }
    E->n_geo = E->geo_off.back();
    E->n_rij = E->rij_off.back();
    if (n == 0) return E.release();
    cudaStream_t const s = L->stream;
    DevBuf<std::uint32_t> ty;
    DevBuf<std::uint8_t> fz;
    ty.reserve(static_cast<std::size_t>(n));
    fz.reserve(static_cast<std::size_t>(n));
    FLY_CUDA(cudaMemcpyAsync(ty.p, h_types, sizeof(std::uint32_t) * static_cast<std::size_t>(n), cudaMemcpyHostToDevice, s));
    FLY_CUDA(cudaMemcpyAsync(fz.p, h_frozen, static_cast<std::size_t>(n), cudaMemcpyHostToDevice, s));
    // offsets with a sentinel: offs[n] = total neighbours
    DevBuf<long long> offs1, goff, roff;
    offs1.reserve(static_cast<std::size_t>(n) + 1);
    goff.reserve(static_cast<std::size_t>(n) + 1);
    roff.reserve(static_cast<std::size_t>(n) + 1);
    FLY_CUDA(cudaMemcpyAsync(offs1.p, offs.p, sizeof(long long) * static_cast<std::size_t>(n), cudaMemcpyDeviceToDevice, s));
    long long const total = nb;
    FLY_CUDA(cudaMemcpyAsync(offs1.p + n, &total, sizeof(long long), cudaMemcpyHostToDevice, s));
    FLY_CUDA(cudaMemcpyAsync(goff.p, E->geo_off.data(), sizeof(long long) * (static_cast<std::size_t>(n) + 1),
                             cudaMemcpyHostToDevice, s));
    FLY_CUDA(cudaMemcpyAsync(roff.p, E->rij_off.data(), sizeof(long long) * (static_cast<std::size_t>(n) + 1),
                             cudaMemcpyHostToDevice, s));
    E->pos.reserve(static_cast<std::size_t>(3 * E->n_geo));
    E->colour.reserve(static_cast<std::size_t>(E->n_geo));
    E->index.reserve(static_cast<std::size_t>(E->n_geo));
    E->r0j.reserve(static_cast<std::size_t>(std::max<std::int64_t>(E->n_geo - n, 1)));
    E->rij.reserve(static_cast<std::size_t>(std::max<std::int64_t>(E->n_rij, 1)));
    launch(k_env_geo, static_cast<unsigned>((n + 127) / 128), 128, 0, s, n, offs1.p, idx.p, dr.p, ty.p, fz.p, E->pos.p,
           E->colour.p, E->index.p);
    // per call and on the current device (cheap; no shared state between host threads)
    FLY_CUDA(cudaFuncSetAttribute(k_env_fp, cudaFuncAttributeMaxDynamicSharedMemorySize, SORT_CAP * sizeof(double)));
    int smax = 1;
    for (std::int64_t i = 0; i < n; ++i) {
      std::int64_t const c = cnt[static_cast<std::size_t>(i)];
      std::int64_t const m = std::max<std::int64_t>(c, c * (c - 1) / 2);
      while (smax < m) smax <<= 1;
    }
    launch(k_env_fp, static_cast<unsigned>(n), 256, static_cast<std::size_t>(smax) * sizeof(double), s, n, goff.p, roff.p,
           E->pos.p, E->r0j.p, E->rij.p);
    FLY_CUDA(cudaStreamSynchronize(s));
    return E.release();
  }

}  // namespace flygpu

namespace {

  template <typename F>
  int env_guard(F&& f) {
    try {
      f();
      return FLYGPU_OK;
    } catch (flygpu::Error const& e) {
      flygpu::set_error(e.msg);
      return e.status;
    } catch (std::bad_alloc const&) {
      flygpu::set_error("host allocation failed");
      return FLYGPU_OOM;
    } catch (std::exception const& e) {
      flygpu::set_error(e.what());
      return FLYGPU_INVALID_ARG;
    }
  }

}  // namespace

extern "C" {

int flygpu_env_build(flygpu_list* list, double r_env, const uint32_t* types, const uint8_t* frozen, flygpu_env** out) {
  return env_guard([&] {
    if (!list || !out) flygpu::fail(FLYGPU_INVALID_ARG, "null argument");
    if (list->n > 0 && (!types || !frozen)) flygpu::fail(FLYGPU_INVALID_ARG, "types and frozen flags are required");
    *out = flygpu::env_build(list, r_env, types, frozen);
  });
}

int flygpu_env_sizes(const flygpu_env* env, int64_t* n_atoms, int64_t* n_geo, int64_t* n_r0j, int64_t* n_rij) {
  return env_guard([&] {
    if (!env) flygpu::fail(FLYGPU_INVALID_ARG, "null environment set");
    if (n_atoms) *n_atoms = env->n;
    if (n_geo) *n_geo = env->n_geo;
    if (n_r0j) *n_r0j = env->n_geo - env->n;
    if (n_rij) *n_rij = env->n_rij;
  });
}

int flygpu_env_get(const flygpu_env* env, int64_t* geo_offsets, double* geo_pos, int32_t* geo_colour,
                   int32_t* geo_index, int64_t* rij_offsets, double* r0j, double* rij) {
  return env_guard([&] {
    if (!env) flygpu::fail(FLYGPU_INVALID_ARG, "null environment set");
    if (geo_offsets) std::copy(env->geo_off.begin(), env->geo_off.end(), geo_offsets);
    if (rij_offsets) std::copy(env->rij_off.begin(), env->rij_off.end(), rij_offsets);
    if (env->n == 0) return;
    std::size_t const g = static_cast<std::size_t>(env->n_geo);
    if (geo_pos) FLY_CUDA(cudaMemcpy(geo_pos, env->pos.p, sizeof(double) * 3 * g, cudaMemcpyDeviceToHost));
    if (geo_colour) FLY_CUDA(cudaMemcpy(geo_colour, env->colour.p, sizeof(int) * g, cudaMemcpyDeviceToHost));
    if (geo_index) FLY_CUDA(cudaMemcpy(geo_index, env->index.p, sizeof(int) * g, cudaMemcpyDeviceToHost));
    if (r0j && g > static_cast<std::size_t>(env->n))
      FLY_CUDA(cudaMemcpy(r0j, env->r0j.p, sizeof(double) * (g - static_cast<std::size_t>(env->n)), cudaMemcpyDeviceToHost));
    if (rij && env->n_rij > 0)
      FLY_CUDA(cudaMemcpy(rij, env->rij.p, sizeof(double) * static_cast<std::size_t>(env->n_rij), cudaMemcpyDeviceToHost));
  });
}

void flygpu_env_destroy(flygpu_env* env) { delete env; }

}  // extern "C"
