// minimise.cu -- LBFGS::minimise for one large system with every vector resident on the device.
//
// Restates src/minimise/LBFGS/lbfgs.cpp:29-115 (trust-radius L-BFGS with the skin rebuild rule) and
// StepLBFGS::newton_step_impl (src/minimise/LBFGS/lbfgs_core.cpp:29-87) for the whole-system relaxation
// an SKMC step ends with (kinetic/skmc.hpp:297-307), over this library's List and EAM. Positions,
// gradients and the m history pairs live in HBM; dot products are two-stage reductions in a fixed order
// (deterministic), and the two-loop recursion's scalars (rho, alpha, beta, the H0 scale) stay in device
// memory, so a step's vector algebra runs without host round trips. The host reads back only what
// LBFGS::minimise branches on: |g|^2 (convergence), |h|^2 (trust scaling and the skin rule) and g.h
// (trust update).

#include <cmath>
#include <vector>

#include "internal.hpp"

namespace flygpu {

  namespace {

    constexpr int RT = 256;   // threads of the vector kernels
    constexpr int RB = 1184;  // blocks of the first reduction stage (a fixed count: a fixed summation order)

    __device__ inline double block_reduce(double v, double* sh) {
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      int const lane = threadIdx.x & 31, w = threadIdx.x >> 5;
      if (lane == 0) sh[w] = v;
      __syncthreads();
      double s = 0;
      if (threadIdx.x == 0)
        for (int k = 0; k < RT / 32; ++k) s += sh[k];
      __syncthreads();
      return s;
    }

    __global__ void __launch_bounds__(RT) k_dot_part(double const* __restrict__ a, double const* __restrict__ b,
                                                     std::int64_t n, double* __restrict__ part) {
      __shared__ double sh[RT / 32];
      double s = 0;
      for (std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * RT + threadIdx.x; i < n;
           i += static_cast<std::int64_t>(gridDim.x) * RT)
        s += a[i] * b[i];
      s = block_reduce(s, sh);
      if (threadIdx.x == 0) part[blockIdx.x] = s;
    }

    __global__ void __launch_bounds__(RT) k_dot_fin(double const* __restrict__ part, int nb, double* __restrict__ out) {
      __shared__ double sh[RT / 32];
      double s = 0;
      for (int i = threadIdx.x; i < nb; i += RT) s += part[i];
      s = block_reduce(s, sh);
      if (threadIdx.x == 0) *out = s;
    }

    // s_p = x - px, y_p = g - pg; then px = x, pg = g, out = g (lbfgs_core.cpp:40-55).
    __global__ void k_pair(double const* __restrict__ x, double* __restrict__ px, double const* __restrict__ g,
                           double* __restrict__ pg, double* __restrict__ sp, double* __restrict__ yp,
                           double* __restrict__ out, std::int64_t n, int have_prev) {
      for (std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * RT + threadIdx.x; i < n;
           i += static_cast<std::int64_t>(gridDim.x) * RT) {
        if (have_prev) {
          sp[i] = x[i] - px[i];
          yp[i] = g[i] - pg[i];
        }
        px[i] = x[i];
        pg[i] = g[i];
        out[i] = g[i];
      }
    }

    __global__ void k_rho(double const* __restrict__ sy, double* __restrict__ rho) { *rho = 1.0 / fabs(*sy); }

    // out -= (rho * dot) y; alpha = rho * dot
    __global__ void k_axpy_alpha(double* __restrict__ out, double const* __restrict__ y, std::int64_t n,
                                 double const* __restrict__ rho, double const* __restrict__ dot,
                                 double* __restrict__ alpha) {
      double const a = *rho * *dot;
      if (blockIdx.x == 0 && threadIdx.x == 0) *alpha = a;
      for (std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * RT + threadIdx.x; i < n;
           i += static_cast<std::int64_t>(gridDim.x) * RT)
        out[i] -= a * y[i];
    }

    // out *= 1 / rho_p / (y_p . y_p)
    __global__ void k_h0(double* __restrict__ out, std::int64_t n, double const* __restrict__ rho,
                         double const* __restrict__ yy) {
      double const sc = 1.0 / *rho / *yy;
      for (std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * RT + threadIdx.x; i < n;
           i += static_cast<std::int64_t>(gridDim.x) * RT)
        out[i] = out[i] * sc;
    }

    // out += (alpha - rho * dot) s
    __global__ void k_axpy_beta(double* __restrict__ out, double const* __restrict__ s, std::int64_t n,
                                double const* __restrict__ rho, double const* __restrict__ dot,
                                double const* __restrict__ alpha) {
      double const c = *alpha - *rho * *dot;
      for (std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * RT + threadIdx.x; i < n;
           i += static_cast<std::int64_t>(gridDim.x) * RT)
        out[i] += c * s[i];
    }

    __global__ void k_scale(double* __restrict__ v, std::int64_t n, double c) {
      for (std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * RT + threadIdx.x; i < n;
           i += static_cast<std::int64_t>(gridDim.x) * RT)
        v[i] *= c;
    }

    __global__ void k_sub(double* __restrict__ x, double const* __restrict__ h, std::int64_t n) {
      for (std::int64_t i = static_cast<std::int64_t>(blockIdx.x) * RT + threadIdx.x; i < n;
           i += static_cast<std::int64_t>(gridDim.x) * RT)
        x[i] -= h[i];
    }

    void ok(int st, char const* what) {
      if (st != FLYGPU_OK) fail(st, std::string(what) + ": " + flygpu_last_error());
    }

    struct Minimiser {
      flygpu_eam* eam;
      int precision;
      cudaStream_t s;
      std::int64_t n3;
      unsigned vb;  // blocks of the vector kernels
      DevBuf<double> part, scal;  // reduction partials; device scalars: [0] dot, [1..m] rho, [m+1..2m] alpha
      PinnedBuf<double> h;
      int m;

      double* dot_dev() { return scal.p; }
      double* rho(int j) { return scal.p + 1 + j; }
      double* alpha(int j) { return scal.p + 1 + m + j; }

      void dot(double const* a, double const* b, double* out) {
        launch(k_dot_part, RB, RT, 0, s, a, b, n3, part.p);
        launch(k_dot_fin, 1, RT, 0, s, part.p, RB, out);
      }
      double dot_host(double const* a, double const* b) {
        dot(a, b, scal.p);
        FLY_CUDA(cudaMemcpyAsync(h.p, scal.p, sizeof(double), cudaMemcpyDeviceToHost, s));
        FLY_CUDA(cudaStreamSynchronize(s));
        return h.p[0];
      }
    };

  }  // namespace

  void minimise_device(flygpu_eam* eam, flygpu_lbfgs_options const& lo, int precision, std::int64_t n,
                       double const* h_pos, std::uint32_t const* h_types, std::uint8_t const* h_frozen,
                       double const ext[3], int const per[3], void* stream, double* h_pos_out,
                       flygpu_search_result& r) {
    if (n <= 0 || !h_pos || !h_types || !h_frozen) fail(FLYGPU_INVALID_ARG, "empty system or null inputs");
    if (lo.n < 1 || lo.n > 1024) fail(FLYGPU_INVALID_ARG, "L-BFGS history length must be 1..1024");
    Minimiser M{};
    M.eam = eam;
    M.precision = precision;
    M.n3 = 3 * n;
    M.m = lo.n;
    bool own = stream == nullptr;
    if (own) {
      FLY_CUDA(cudaStreamCreateWithFlags(&M.s, cudaStreamNonBlocking));
    } else {
      M.s = static_cast<cudaStream_t>(stream);
    }
    struct StreamGuard {
      cudaStream_t s;
      bool own;
      ~StreamGuard() {
        if (own && s) {
          cudaStreamSynchronize(s);
          cudaStreamDestroy(s);
        }
      }
    } guard_s{M.s, own};
    M.vb = static_cast<unsigned>(std::min<std::int64_t>((M.n3 + RT - 1) / RT, 4 * 1184));
    M.part.reserve(RB);
    M.scal.reserve(static_cast<std::size_t>(1 + 2 * M.m));
    M.h.reserve(4);
    std::size_t const N = static_cast<std::size_t>(M.n3);
    DevBuf<double> x, g, px, pg, out, S, Y, e;
    DevBuf<std::uint32_t> ty;
    DevBuf<std::uint8_t> fz;
    x.reserve(N);
    g.reserve(N);
    px.reserve(N);
    pg.reserve(N);
    out.reserve(N);
    S.reserve(N * static_cast<std::size_t>(M.m));
    Y.reserve(N * static_cast<std::size_t>(M.m));
    e.reserve(1);
    ty.reserve(static_cast<std::size_t>(n));
    fz.reserve(static_cast<std::size_t>(n));
    FLY_CUDA(cudaMemcpyAsync(x.p, h_pos, sizeof(double) * N, cudaMemcpyHostToDevice, M.s));
    FLY_CUDA(cudaMemcpyAsync(ty.p, h_types, sizeof(std::uint32_t) * static_cast<std::size_t>(n), cudaMemcpyHostToDevice, M.s));
    FLY_CUDA(cudaMemcpyAsync(fz.p, h_frozen, static_cast<std::size_t>(n), cudaMemcpyHostToDevice, M.s));
    // the list: LBFGS::minimise's cut-off r_cut + skin (lbfgs.cpp:41-45)
    double const rc = eam->r_cut;
    double const skin = std::max(std::pow(lo.skin_frac, 1. / 3.) - 1, 0.0) * rc;
    flygpu_list* L = nullptr;
    ok(flygpu_list_create(ext, per, rc + skin, M.s, &L), "List");
    struct ListGuard {
      flygpu_list* L;
      ~ListGuard() { flygpu_list_destroy(L); }
    } guard_l{L};
    auto rebuild = [&] { ok(flygpu_list_rebuild_device(L, x.p, n), "List::rebuild"); };
    bool types_sent = false;
    long long grad_calls = 0;
    auto gradient = [&](double* d_e) {
      ok(flygpu_eam_energy_gradient_device(eam, L, types_sent ? nullptr : ty.p, types_sent ? nullptr : fz.p, precision,
                                           d_e, g.p),
         "EAM::gradient");
      types_sent = true;
      ++grad_calls;
    };
    auto step = [&](int k) {  // StepLBFGS::newton_step_impl into out; k = calls so far
      int const prev = k > 0 ? (k - 1) % M.m : 0;
      double* sp = S.p + N * static_cast<std::size_t>(prev);
      double* yp = Y.p + N * static_cast<std::size_t>(prev);
      launch(k_pair, M.vb, RT, 0, M.s, x.p, px.p, g.p, pg.p, sp, yp, out.p, M.n3, k > 0 ? 1 : 0);
      if (k > 0) {
        M.dot(sp, yp, M.dot_dev());
        launch(k_rho, 1, 1, 0, M.s, M.dot_dev(), M.rho(prev));
      }
      int const incur = k <= M.m ? 0 : k - M.m, bound = k <= M.m ? k : M.m;
      for (int i = bound - 1; i >= 0; --i) {
        int const j = (i + incur) % M.m;
        double const* sj = S.p + N * static_cast<std::size_t>(j);
        double const* yj = Y.p + N * static_cast<std::size_t>(j);
        M.dot(sj, out.p, M.dot_dev());
        launch(k_axpy_alpha, M.vb, RT, 0, M.s, out.p, yj, M.n3, M.rho(j), M.dot_dev(), M.alpha(j));
      }
      if (k > 0) {
        M.dot(yp, yp, M.dot_dev());
        launch(k_h0, M.vb, RT, 0, M.s, out.p, M.n3, M.rho(prev), M.dot_dev());
      }
      for (int i = 0; i <= bound - 1; ++i) {
        int const j = (i + incur) % M.m;
        double const* sj = S.p + N * static_cast<std::size_t>(j);
        double const* yj = Y.p + N * static_cast<std::size_t>(j);
        M.dot(yj, out.p, M.dot_dev());
        launch(k_axpy_beta, M.vb, RT, 0, M.s, out.p, sj, M.n3, M.rho(j), M.dot_dev(), M.alpha(j));
      }
    };
    rebuild();
    gradient(nullptr);
    double trust = lo.min_trust, acc = 0;
    int i = 0, k = 0;
    r = flygpu_search_result{};
    r.exit_code = 1;  // LBFGS::minimise returns true (failure) unless it converges
    for (; i < lo.iter_max; ++i) {
      if (M.dot_host(g.p, g.p) < lo.f2norm * lo.f2norm) {
        r.exit_code = 0;
        break;
      }
      step(k++);
      double const hh = M.dot_host(out.p, out.p);
      double const sc = std::min(1.0, trust / std::sqrt(hh));
      launch(k_scale, M.vb, RT, 0, M.s, out.p, M.n3, sc);
      acc += std::sqrt(M.dot_host(out.p, out.p));
      launch(k_sub, M.vb, RT, 0, M.s, x.p, out.p, M.n3);
      if (acc > 0.5 * skin) {
        rebuild();
        acc = 0;
      } else {
        ok(flygpu_list_update_device(L, out.p), "List::update");
      }
      gradient(nullptr);
      double const proj = M.dot_host(g.p, out.p);
      if (proj < -lo.proj_tol) {
        trust = std::max(lo.min_trust, lo.shrink_trust * trust);
      } else if (proj > lo.proj_tol) {
        trust = std::min(lo.max_trust, lo.grow_trust * trust);
      }
    }
    r.steps = i;
    rebuild();
    gradient(e.p);
    --grad_calls;  // the energy evaluation at the end is not one of the minimiser's gradient calls
    FLY_CUDA(cudaMemcpyAsync(M.h.p, e.p, sizeof(double), cudaMemcpyDeviceToHost, M.s));
    if (h_pos_out) FLY_CUDA(cudaMemcpyAsync(h_pos_out, x.p, sizeof(double) * N, cudaMemcpyDeviceToHost, M.s));
    FLY_CUDA(cudaStreamSynchronize(M.s));
    r.energy = M.h.p[0];
    r.grad_calls = grad_calls;
    r.status = FLYGPU_OK;
  }

}  // namespace flygpu

extern "C" int flygpu_minimise(flygpu_eam* eam, const flygpu_lbfgs_options* lbfgs, int precision, int64_t n,
                               const double* pos, const uint32_t* types, const uint8_t* frozen, const double extents[3],
                               const int periodic[3], void* stream, double* pos_out, flygpu_search_result* result) {
  try {
    if (!eam || !result || !extents || !periodic) flygpu::fail(FLYGPU_INVALID_ARG, "null argument");
    flygpu_lbfgs_options l;
    flygpu_lbfgs_options_default(&l);
    if (lbfgs) l = *lbfgs;
    flygpu::minimise_device(eam, l, precision, n, pos, types, frozen, extents, periodic, stream, pos_out, *result);
    return FLYGPU_OK;
  } catch (flygpu::Error const& e) {
    flygpu::set_error(e.msg);
    return e.status;
  } catch (std::exception const& e) {
    flygpu::set_error(e.what());
    return FLYGPU_INVALID_ARG;
  }
}
