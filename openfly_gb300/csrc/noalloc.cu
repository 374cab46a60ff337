// noalloc.cu -- EAM energy + gradient for callers that cannot allocate device memory.
//
// Some callers cannot call cudaMalloc: code running inside another framework's memory manager that
// owns every device allocation, a pre-allocated real-time loop that must not touch the allocator
// after start-up, or a caller holding only borrowed device pointers. flygpu_eam_energy_gradient_noalloc
// serves them: it takes device inputs and outputs from the caller and keeps its scratch (the per-atom
// F'(rho), block partial energies and an error word) in one file-scope __device__ array of fixed size,
// so the call itself allocates nothing. The array is sized for FLYGPU_NOALLOC_MAX_ATOMS atoms and every
// GPU that loads the library holds it until the process exits.
//
// The pair search is an O(n^2) minimum-image scan (no neighbour list, so nothing to allocate), which
// visits the same pairs as List::for_neighbours (neigh/list.hpp:139-154) when every periodic extent
// exceeds twice the cut-off; the arithmetic is EAM::energy / EAM::gradient's in binary64
// (src/potential/EAM/eam.cpp:33-120), compiled with -fmad=false.

#include <mutex>

#include "internal.hpp"

namespace {

  constexpr int T = 128;
  constexpr int MAX_BLOCKS = (FLYGPU_NOALLOC_MAX_ATOMS + T - 1) / T;
  // scratch layout, in doubles: F'(rho) per atom, two partial sums per block, one error word
  constexpr int OFF_PART = FLYGPU_NOALLOC_MAX_ATOMS;
  constexpr int OFF_ERR = OFF_PART + 2 * MAX_BLOCKS;
  constexpr int SCRATCH_DOUBLES = OFF_ERR + 32;

  static __device__ __align__(256) double g_noalloc_scratch[SCRATCH_DOUBLES];

  using flygpu::D4;
  using flygpu::TablesView;

  struct Box {
    double L[3], inv[3];
    int per[3];
  };

  __device__ inline void min_image(Box const& b, double& dx, double& dy, double& dz) {
    if (b.per[0]) dx -= b.L[0] * rint(dx * b.inv[0]);
    if (b.per[1]) dy -= b.L[1] * rint(dy * b.inv[1]);
    if (b.per[2]) dz -= b.L[2] * rint(dz * b.inv[2]);
  }

  __device__ inline bool lookup(double x, double inv_dx, double dx, int n, long long& i, double& x0) {
    if (!(x >= 0)) return false;
    double const u = x * inv_dx;
    if (!(u < static_cast<double>(n))) return false;
    i = static_cast<long long>(u);
    x0 = x - static_cast<double>(i) * dx;
    return true;
  }

  __device__ inline double val(D4 const& c, double x0) { return c.x + x0 * (c.y + x0 * (c.z + x0 * c.w)); }
  __device__ inline double der(D4 const& c, double x0) { return c.y + x0 * (2.0 * c.z + x0 * 3.0 * c.w); }

  __device__ double block_sum(double v) {
    __shared__ double sh[T / 32];
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = v;
    __syncthreads();
    double s = 0;
    if (threadIdx.x == 0)
      for (int w = 0; w < T / 32; ++w) s += sh[w];
    __syncthreads();
    return s;
  }

  __device__ inline int type_of(std::uint32_t const* types, int i, int nt, int* err) {
    std::uint32_t const t = types[i];
    if (t >= static_cast<std::uint32_t>(nt)) {
      atomicOr(err, flygpu::ERR_BAD_INDEX);
      return 0;
    }
    return static_cast<int>(t);
  }

  // rho_i, F'(rho_i) into scratch, per-block partial sums of v and F for the energy.
  __global__ void __launch_bounds__(T) k_density(TablesView tb, double const* __restrict__ pos,
                                                 std::uint32_t const* __restrict__ types, int n, Box box, double rc2,
                                                 double* __restrict__ scratch) {
    int const i = blockIdx.x * T + threadIdx.x;
    int* err = reinterpret_cast<int*>(scratch + OFF_ERR);
    double vs = 0, fe = 0;
    if (i < n) {
      int const nt = tb.n_types;
      int const ti = type_of(types, i, nt, err);
      double const xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
      double rho = 0;
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        double dx = pos[3 * j] - xi, dy = pos[3 * j + 1] - yi, dz = pos[3 * j + 2] - zi;
        min_image(box, dx, dy, dz);
        double const r2 = (dx * dx + dy * dy) + dz * dz;
        if (r2 < rc2) {
          int const tj = type_of(types, j, nt, err);
          long long k;
          double x0;
          if (!lookup(sqrt(r2), tb.inv_dR, tb.dR, tb.nR, k, x0)) {
            atomicOr(err, flygpu::ERR_SPLINE_OOB);
            continue;
          }
          vs += val(tb.v64[static_cast<long long>(ti + nt * tj) * tb.nR + k], x0);
          rho += val(tb.phi64[static_cast<long long>(tj + nt * ti) * tb.nR + k], x0);
        }
      }
      long long k;
      double x0;
      double fp = 0;
      if (lookup(rho, tb.inv_dP, tb.dP, tb.nP, k, x0)) {
        D4 const c = tb.F64[static_cast<long long>(ti) * tb.nP + k];
        fp = der(c, x0);
        fe = val(c, x0);
      } else {
        atomicOr(err, flygpu::ERR_SPLINE_OOB);
      }
      scratch[i] = fp;
    }
    double const a = block_sum(vs), b = block_sum(fe);
    if (threadIdx.x == 0) {
      scratch[OFF_PART + 2 * blockIdx.x] = a;
      scratch[OFF_PART + 2 * blockIdx.x + 1] = b;
    }
  }

  __global__ void __launch_bounds__(T) k_force(TablesView tb, double const* __restrict__ pos,
                                               std::uint32_t const* __restrict__ types,
                                               std::uint8_t const* __restrict__ frozen, int n, Box box, double rc2,
                                               double const* __restrict__ scratch, double* __restrict__ grad) {
    int const i = blockIdx.x * T + threadIdx.x;
    if (i >= n) return;
    int* err = reinterpret_cast<int*>(const_cast<double*>(scratch) + OFF_ERR);
    double gx = 0, gy = 0, gz = 0;
    if (!frozen[i]) {
      int const nt = tb.n_types;
      int const ti = type_of(types, i, nt, err);
      double const xi = pos[3 * i], yi = pos[3 * i + 1], zi = pos[3 * i + 2];
      double const fpi = scratch[i];
      for (int j = 0; j < n; ++j) {
        if (j == i) continue;
        double dx = pos[3 * j] - xi, dy = pos[3 * j + 1] - yi, dz = pos[3 * j + 2] - zi;
        min_image(box, dx, dy, dz);
        double const r2 = (dx * dx + dy * dy) + dz * dz;
        if (r2 < rc2) {
          int const tj = type_of(types, j, nt, err);
          double const r = sqrt(r2);
          long long k;
          double x0;
          if (!lookup(r, tb.inv_dR, tb.dR, tb.nR, k, x0)) {
            atomicOr(err, flygpu::ERR_SPLINE_OOB);
            continue;
          }
          double const mag = der(tb.v64[static_cast<long long>(tj + nt * ti) * tb.nR + k], x0) +
                             fpi * der(tb.phi64[static_cast<long long>(tj + nt * ti) * tb.nR + k], x0) +
                             scratch[j] * der(tb.phi64[static_cast<long long>(ti + nt * tj) * tb.nR + k], x0);
          double const s = mag / r;
          gx -= s * dx;
          gy -= s * dy;
          gz -= s * dz;
        }
      }
    }
    grad[3 * i] = gx;
    grad[3 * i + 1] = gy;
    grad[3 * i + 2] = gz;
  }

  __global__ void k_energy(double const* __restrict__ scratch, int nblocks, double* __restrict__ energy) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double v = 0, f = 0;
    for (int b = 0; b < nblocks; ++b) {
      v += scratch[OFF_PART + 2 * b];
      f += scratch[OFF_PART + 2 * b + 1];
    }
    *energy = (0.5 * v) + f;
  }

  // Device address of the scratch array, looked up once per device (cudaGetSymbolAddress with that
  // device current) and cached.
  std::mutex g_mu;
  double* g_ptr[256] = {};

  double* scratch_for_current_device() {
    int dev = 0;
    FLY_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 256) flygpu::fail(FLYGPU_INVALID_ARG, "device index out of range");
    std::lock_guard<std::mutex> lk(g_mu);
    if (!g_ptr[dev]) {
      void* p = nullptr;
      cudaError_t const e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
      if (e != cudaSuccess) flygpu::fail(FLYGPU_CUDA_ERROR, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
      g_ptr[dev] = static_cast<double*>(p);
    }
    return g_ptr[dev];
  }

}  // namespace

extern "C" int flygpu_eam_energy_gradient_noalloc(const flygpu_eam* eam, const double* d_pos,
                                                  const uint32_t* d_types, const uint8_t* d_frozen, int64_t n,
                                                  const double extents[3], const int periodic[3], double* d_energy,
                                                  double* d_grad, void* stream) {
  try {
    if (!eam || !d_pos || !d_types || !d_frozen || !extents || !periodic || !d_energy || !d_grad)
      flygpu::fail(FLYGPU_INVALID_ARG, "null argument");
    if (n < 1 || n > FLYGPU_NOALLOC_MAX_ATOMS)
      flygpu::fail(FLYGPU_INVALID_ARG, "flygpu_eam_energy_gradient_noalloc takes 1.." +
                                           std::to_string(FLYGPU_NOALLOC_MAX_ATOMS) + " atoms, got " +
                                           std::to_string(n));
    double const rc = eam->r_cut;
    Box box{};
    for (int k = 0; k < 3; ++k) {
      if (!(extents[k] > 0)) flygpu::fail(FLYGPU_INVALID_ARG, "box extents must be positive");
      box.L[k] = extents[k];
      box.inv[k] = 1.0 / extents[k];
      box.per[k] = periodic[k] ? 1 : 0;
      if (box.per[k] && !(extents[k] > 2 * rc))
        flygpu::fail(FLYGPU_INVALID_ARG, "periodic extents must exceed twice the cut-off");
    }
    cudaStream_t const s = static_cast<cudaStream_t>(stream);
    double* scratch = scratch_for_current_device();
    int const nb = static_cast<int>((n + T - 1) / T);
    FLY_CUDA(cudaMemsetAsync(scratch + OFF_ERR, 0, sizeof(int), s));
    TablesView const tb = eam->view();
    double const rc2 = rc * rc;
    flygpu::launch(k_density, nb, T, 0, s, tb, d_pos, d_types, static_cast<int>(n), box, rc2, scratch);
    flygpu::launch(k_force, nb, T, 0, s, tb, d_pos, d_types, d_frozen, static_cast<int>(n), box, rc2,
                   static_cast<double const*>(scratch), d_grad);
    flygpu::launch(k_energy, 1, 32, 0, s, static_cast<double const*>(scratch), nb, d_energy);
    int err = 0;
    FLY_CUDA(cudaMemcpyAsync(&err, scratch + OFF_ERR, sizeof(int), cudaMemcpyDeviceToHost, s));
    FLY_CUDA(cudaStreamSynchronize(s));
    if (err) {
      int const st = flygpu::status_from_word(err);
      flygpu::fail(st, st == FLYGPU_SPLINE_OOB ? "spline argument outside the tabulated region" : "type index out of range");
    }
    return FLYGPU_OK;
  } catch (flygpu::Error const& e) {
    flygpu::set_error(e.msg);
    return e.status;
  }
}
