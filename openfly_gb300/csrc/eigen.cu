// eigen.cu -- eigenvalues of a dense symmetric binary64 matrix on the device (the prefactor step's
// Hessian::eigenvalues, system/hessian.hpp:86-93, which the reference hands to Eigen's
// SelfAdjointEigenSolver: Householder tridiagonalisation, then the tridiagonal's eigenvalues).
//
// Stage 1, k_tridiag: Householder reduction to tridiagonal form by one thread-block cluster (16 CTAs
// where the GPU allows it, else 8, 4, ...). CTA c owns the rows i with i mod C == c and keeps them in its
// shared memory when they fit (ceil(M / C) rows: 66 KB a CTA for M = 342), else in the global matrix.
// Step k, for the trailing block below row k:
//   every CTA reads row k (from its owner's shared memory) and forms the same reflector:
//   alpha = -sign(x0) |x| for x = A[k, k+1:], u = x - alpha e1, tau = 1 / (alpha^2 - alpha x0), so
//   H = I - tau u u^T maps x to alpha e1;
//   owned rows: p_i = tau sum_j A[i, j] u_j, and the CTA's share of u^T p;
//   cluster barrier;
//   every CTA: K = tau / 2 sum (u^T p), w = p - K u (p read from the owners' shared memory);
//   owned rows: A[i, j] -= u_i w_j + w_i u_j;
//   cluster barrier.
// d_k = A[k, k], e_k = alpha. Every CTA runs the same loop with the same trip count and no early exit, so
// every barrier is reached by all of them (hardware cluster barriers, not spin loops). On the global path
// the rows are read with ld.global.cg (L2, not L1) after the barriers' release/acquire.
// GB300 issues binary64 at about 1/64 of the binary32 rate and a dependent binary64 operation takes ~67
// cycles, so the kernel spends binary64 instructions only where they carry the algorithm: reductions
// run on the warps that hold data, the update is two fused multiply-adds an element, and rows are
// walked in full groups of four plus a one-wide tail (no masked lanes).
// Stage 2, k_bisect: the tridiagonal's eigenvalues by Sturm-sequence multisection, one warp per
// eigenvalue index j: the 32 lanes count the eigenvalues below 32 points of the current interval (sign
// changes of the leading principal minors of T - x I, a division-free three-term recurrence), the
// interval shrinks to the sub-interval holding eigenvalue j, and the loop stops when it is within 4 ulp
// of its endpoints or of 2 eps |T|. Ascending order comes from j.

#include <cooperative_groups.h>

#include <algorithm>
#include <cfloat>
#include <cmath>

#include "internal.hpp"

namespace cg = cooperative_groups;

namespace flygpu {

  namespace {

    constexpr int TT = 512;  // threads per CTA of k_tridiag
    constexpr int TW = TT / 32;
    constexpr int TRIDIAG_SMEM_MAX = 220 * 1024;  // dynamic shared memory limit set on k_tridiag

    // sqrt(a) and 1 / a from binary32 seeds and Newton steps in binary64 (each a short chain of FMAs;
    // the correctly rounded library forms are long dependent chains at 67 cycles a binary64 operation).
    // Accurate to a few ulp for a in the binary32 exponent range, which the caller checks.
    __device__ inline double fast_rsqrt(double a) {
      double y = static_cast<double>(rsqrtf(static_cast<float>(a)));
      double const h = 0.5 * a;
      y = y * fma(-h * y, y, 1.5);
      y = y * fma(-h * y, y, 1.5);
      return y * fma(-h * y, y, 1.5);
    }
    __device__ inline double fast_rcp(double a) {
      double y = static_cast<double>(__frcp_rn(static_cast<float>(a)));
      y = y * fma(-a, y, 2.0);
      y = y * fma(-a, y, 2.0);
      return y * fma(-a, y, 2.0);
    }
    __device__ inline bool f32_range(double a) { return a > 1e-30 && a < 1e30; }

    // Sum over the CTA of v, where only warps w < nw hold data: their lanes reduce with shuffles, their
    // leaders' sums are added by warp 0 (binary64 adds are the scarce resource; idle warps add nothing).
    __device__ double cta_sum(double v, double* red, int nw) {
      int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      if (warp < nw) {
        for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
        if (lane == 0) red[warp] = v;
      }
      __syncthreads();
      if (warp == 0) {
        double t = lane < nw ? red[lane] : 0.0;
        for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
        if (lane == 0) red[TW] = t;
      }
      __syncthreads();
      double const s = red[TW];
      __syncthreads();
      return s;
    }

    // The rows of the matrix a CTA owns: in its shared memory (SM) or in the global matrix.
    template <bool SM>
    struct Rows {
      double* base;  // SM: the CTA's rows, local row r at base + r M; else the global matrix
      int M, C;
      __device__ double* own(int i) const {
        return SM ? base + static_cast<std::int64_t>(i / C) * M : base + static_cast<std::int64_t>(i) * M;
      }
    };

    template <bool SM>
    __device__ inline double ld(double const* p) {
      if constexpr (SM) {
        return *p;
      } else {
        return __ldcg(p);
      }
    }
    template <bool SM>
    __device__ inline void st(double* p, double v) {
      if constexpr (SM) {
        *p = v;
      } else {
        __stcg(p, v);
      }
    }

    // Householder tridiagonalisation of the M x M symmetric A (full storage; overwritten on the global
    // path). d: M, e: M (e[M-1] unused). Launched as one cluster of C CTAs; CTA c owns the rows i with
    // i mod C == c. With SM every CTA keeps its rows in shared memory (ceil(M / C) rows). Row k, the p
    // values and the CTAs' shares of u^T p are read across the cluster through distributed shared memory.
    template <bool SM>
    __global__ void __launch_bounds__(TT) k_tridiag(double* __restrict__ A, int M, double* __restrict__ d,
                                                   double* __restrict__ e) {
      cg::cluster_group cl = cg::this_cluster();
      int const C = static_cast<int>(cl.num_blocks());
      int const c = static_cast<int>(cl.block_rank());
      int const R = (M + C - 1) / C;
      extern __shared__ double sm[];
      double* rows = sm;                                              // SM: R x M
      double* u = sm + (SM ? static_cast<std::int64_t>(R) * M : 0);  // M
      double* w = u + M;                                              // M
      double* pl = w + M;                                             // M: p_i of the owned rows, at index i
      double* share = pl + M;                                         // 1
      double* red = share + 1;                                        // TW + 1
      int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      Rows<SM> const own{SM ? rows : A, M, C};
      if (SM) {
        for (int r = warp; r * C + c < M; r += TW)
          for (int j = lane; j < M; j += 32)
            rows[static_cast<std::int64_t>(r) * M + j] = __ldcg(A + static_cast<std::int64_t>(r * C + c) * M + j);
        cl.sync();
      }
      for (int k = 0; k + 2 < M; ++k) {
        int const b = k + 1, m = M - b;
        double const* rk = SM ? cl.map_shared_rank(rows, k % C) + static_cast<std::int64_t>(k / C) * M
                              : A + static_cast<std::int64_t>(k) * M;
        double s2 = 0;
        for (int j = threadIdx.x; j < m; j += TT) {
          double const x = ld<SM>(rk + b + j);
          u[j] = x;
          s2 = fma(x, x, s2);
        }
        s2 = cta_sum(s2, red, min(TW, (m + 31) / 32));
        double const x0 = u[0];
        double const nrm = f32_range(s2) ? s2 * fast_rsqrt(s2) : sqrt(s2);
        double const alpha = x0 > 0 ? -nrm : nrm;
        double const den = alpha * alpha - alpha * x0;
        // a column that is already zero below the sub-diagonal needs no reflection (tau = 0)
        double const tau = den > 0 && s2 - x0 * x0 > 0 ? (f32_range(den) ? fast_rcp(den) : 1.0 / den) : 0.0;
        __syncthreads();
        if (threadIdx.x == 0) u[0] = tau != 0.0 ? x0 - alpha : 0.0;
        if (c == 0 && threadIdx.x == 0) {
          d[k] = ld<SM>(rk + k);
          e[k] = tau != 0.0 ? alpha : x0;
        }
        __syncthreads();
        // p_i = tau (A u)_i over owned rows, and the share of u^T p. Each lane keeps four independent
        // partial sums (loads in groups of 4), so a row's dependent chain is a quarter of its length.
        double sh = 0;
        for (int r = warp; r * C + c < M; r += TW) {
          int const i = r * C + c;
          if (i < b) continue;
          double const* ri = own.own(i) + b;
          double acc[4] = {0, 0, 0, 0};
          int j = lane;
          for (; j + 96 < m; j += 128) {
            double v[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) v[t] = ld<SM>(ri + j + 32 * t);
#pragma unroll
            for (int t = 0; t < 4; ++t) acc[t] = fma(v[t], u[j + 32 * t], acc[t]);
          }
          for (; j < m; j += 32) acc[0] = fma(ld<SM>(ri + j), u[j], acc[0]);
          double a = (acc[0] + acc[1]) + (acc[2] + acc[3]);
          for (int o = 16; o > 0; o >>= 1) a += __shfl_down_sync(0xffffffffu, a, o);
          if (lane == 0) {
            double const pi = tau * a;
            pl[i] = pi;
            sh = fma(u[i - b], pi, sh);
          }
        }
        // the share: one value per warp leader, summed by warp 0
        if (lane == 0) red[warp] = sh;
        __syncthreads();
        if (warp == 0) {
          double t = lane < TW ? red[lane] : 0.0;
          for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
          if (lane == 0) *share = t;
        }
        cl.sync();
        // K = tau / 2 sum of the CTAs' shares: a shuffle tree in warp 0, broadcast through shared memory
        if (warp == 0) {
          double t = lane < C ? *cl.map_shared_rank(share, lane) : 0.0;
          for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
          if (lane == 0) red[TW] = 0.5 * tau * t;
        }
        __syncthreads();
        double const K = red[TW];
        for (int j = threadIdx.x; j < m; j += TT) w[j] = fma(-K, u[j], cl.map_shared_rank(pl, (b + j) % C)[b + j]);
        __syncthreads();
        for (int r = warp; r * C + c < M; r += TW) {
          int const i = r * C + c;
          if (i < b) continue;
          double* ri = own.own(i) + b;
          double const ui = u[i - b], wi = w[i - b];
          // A_ij - u_i w_j - w_i u_j as two fused multiply-adds
          int j = lane;
          for (; j + 96 < m; j += 128) {
            double v[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) v[t] = ld<SM>(ri + j + 32 * t);
#pragma unroll
            for (int t = 0; t < 4; ++t) st<SM>(ri + j + 32 * t, fma(-ui, w[j + 32 * t], fma(-wi, u[j + 32 * t], v[t])));
          }
          for (; j < m; j += 32) st<SM>(ri + j, fma(-ui, w[j], fma(-wi, u[j], ld<SM>(ri + j))));
        }
        cl.sync();
      }
      if (c == 0 && threadIdx.x == 0) {
        auto at = [&](int i, int j) {
          return SM ? cl.map_shared_rank(rows, i % C)[static_cast<std::int64_t>(i / C) * M + j]
                    : __ldcg(A + static_cast<std::int64_t>(i) * M + j);
        };
        if (M >= 2) {
          d[M - 2] = at(M - 2, M - 2);
          e[M - 2] = at(M - 1, M - 2);
        }
        d[M - 1] = at(M - 1, M - 1);
      }
      cl.sync();  // no CTA leaves while another may still read its shared memory
    }

    // Number of eigenvalues of the tridiagonal (d, e2 = e^2) below x: the sign changes of the sequence
    // 1, p_0, p_1, ... of leading principal minors of T - x I, p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2}
    // (the Sturm sequence; no divisions, which cost dozens of binary64 instructions on this GPU). A zero
    // minor takes the sign opposite to the one before it. Signs, zeros and magnitudes are read from the
    // bit patterns with integer instructions; every 8 minors the last two are rescaled by a power of two
    // when they leave [2^-600, 2^600] (8 steps cannot overflow from there), which keeps every sign.
    __device__ inline bool neg(double v) { return __double_as_longlong(v) < 0; }
    __device__ inline int expo(double v) { return static_cast<int>((__double_as_longlong(v) >> 52) & 0x7ff); }
    __device__ inline bool is_zero(double v) { return (__double_as_longlong(v) << 1) == 0; }

    __device__ int sturm_count(double const* __restrict__ d, double const* __restrict__ e2, int M, double x) {
      double pm = 1.0, p = d[0] - x;
      if (is_zero(p)) p = -0x1p-200;
      int cnt = neg(p);
      for (int i = 1; i < M; ++i) {
        double pn = fma(d[i] - x, p, -(e2[i - 1] * pm));
        if (is_zero(pn)) pn = -p * 0x1p-200;
        cnt += neg(pn) != neg(p);
        pm = p;
        p = pn;
        if ((i & 7) == 0) {
          int const ep = expo(p);
          if (ep > 1023 + 600) {
            p *= 0x1p-600;
            pm *= 0x1p-600;
          } else if (ep < 1023 - 600 && expo(pm) < 1023 - 600) {
            p *= 0x1p600;
            pm *= 0x1p600;
          }
        }
      }
      return cnt;
    }

    // One warp per eigenvalue index; bounds = {lo, hi, tol}.
    __global__ void k_bisect(double const* __restrict__ d, double const* __restrict__ e2, int M,
                             double const* __restrict__ bounds, double* __restrict__ eig) {
      int const lane = threadIdx.x & 31;
      int const j = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
      if (j >= M) return;
      double lo = bounds[0], hi = bounds[1];
      double const tol = bounds[2];
      for (int it = 0; it < 64; ++it) {
        double const width = hi - lo;
        if (width <= fmax(tol, 4 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)))) break;
        double const x = lo + width * (static_cast<double>(lane + 1) * (1.0 / 33.0));
        int const cnt = sturm_count(d, e2, M, x);
        unsigned const above = __ballot_sync(0xffffffffu, cnt > j);
        double const xs = __shfl_sync(0xffffffffu, x, above ? __ffs(above) - 1 : 31);
        if (above == 0u) {
          lo = xs;
        } else {
          int const f = __ffs(above) - 1;
          double const xp = __shfl_sync(0xffffffffu, x, f > 0 ? f - 1 : 0);
          hi = xs;
          if (f > 0) lo = xp;
        }
      }
      if (lane == 0) eig[j] = 0.5 * (lo + hi);
    }

    // out (M x M, full) = the symmetric matrix of the row-major lower triangle of H (N x N) restricted to
    // the coordinates act (all when act is null).
    __global__ void k_sym_gather(double const* __restrict__ H, std::int64_t N, int const* __restrict__ act,
                                 std::int64_t M, double* __restrict__ out) {
      std::int64_t const t = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (t >= M * M) return;
      std::int64_t const r = t / M, q = t - r * M;
      std::int64_t const a = act ? act[r] : r, b = act ? act[q] : q;
      out[t] = a >= b ? H[a * N + b] : H[b * N + a];
    }

    std::size_t tridiag_smem(int M, int C, bool sm) {
      std::size_t const R = sm ? static_cast<std::size_t>((M + C - 1) / C) : 0;
      return (R * static_cast<std::size_t>(M) + 3 * static_cast<std::size_t>(M) + 1 + TW + 1) * sizeof(double);
    }

    cudaLaunchConfig_t tridiag_config(int C, std::size_t smem, cudaLaunchAttribute& at, cudaStream_t s) {
      cudaLaunchConfig_t cfg{};
      cfg.gridDim = dim3(C);
      cfg.blockDim = dim3(TT);
      cfg.dynamicSmemBytes = smem;
      cfg.stream = s;
      at.id = cudaLaunchAttributeClusterDimension;
      at.val.clusterDim.x = C;
      at.val.clusterDim.y = 1;
      at.val.clusterDim.z = 1;
      cfg.attrs = &at;
      cfg.numAttrs = 1;
      return cfg;
    }

    template <bool SM>
    bool tridiag_fits(int M, int C) {
      std::size_t const smem = tridiag_smem(M, C, SM);
      if (smem > static_cast<std::size_t>(TRIDIAG_SMEM_MAX)) return false;
      cudaLaunchAttribute at{};
      cudaLaunchConfig_t const cfg = tridiag_config(C, smem, at, nullptr);
      int n = 0;
      bool const ok = cudaOccupancyMaxActiveClusters(&n, k_tridiag<SM>, &cfg) == cudaSuccess && n > 0;
      cudaGetLastError();
      return ok;
    }

    // Launches the tridiagonalisation of the M x M matrix A (global) on stream s: the largest cluster
    // (16, 8, ... CTAs) the device can hold, with the rows in shared memory when they fit. The kernels'
    // shared-memory limits are set to the same constant on every call, so concurrent callers agree.
    void tridiag_launch(double* A, int M, double* d, double* e, cudaStream_t s) {
      for (auto k : {k_tridiag<true>, k_tridiag<false>}) {
        FLY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, TRIDIAG_SMEM_MAX));
        FLY_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      }
      for (int C : {16, 8, 4, 2, 1}) {
        bool const sm = tridiag_fits<true>(M, C);
        if (!sm && !tridiag_fits<false>(M, C)) continue;
        cudaLaunchAttribute at{};
        cudaLaunchConfig_t const cfg = tridiag_config(C, tridiag_smem(M, C, sm), at, s);
        if (sm) {
          FLY_CUDA(cudaLaunchKernelEx(&cfg, k_tridiag<true>, A, M, d, e));
        } else {
          FLY_CUDA(cudaLaunchKernelEx(&cfg, k_tridiag<false>, A, M, d, e));
        }
        count_launch();
        return;
      }
      fail(FLYGPU_CUDA_ERROR, "no thread-block cluster shape fits the tridiagonalisation kernel");
    }

  }  // namespace

  void dense_eigenvalues(flygpu_list* L, double const* d_H, std::int64_t N, std::vector<int> const& act, double* h_eig) {
    std::int64_t const M = act.empty() ? N : static_cast<std::int64_t>(act.size());
    if (M == 0) return;
    if (M > MAX_DENSE_EIG)
      fail(FLYGPU_INVALID_ARG, "the dense eigensolver takes at most " + std::to_string(MAX_DENSE_EIG) + " coordinates");
    cudaStream_t const s = L->stream;
    HessianScratch& P = L->hs;
    P.sub.reserve(static_cast<std::size_t>(M * M));
    P.tri.reserve(4 * static_cast<std::size_t>(M) + 8);
    int const* d_act = nullptr;
    if (!act.empty()) {
      P.act.reserve(act.size());
      FLY_CUDA(cudaMemcpyAsync(P.act.p, act.data(), sizeof(int) * act.size(), cudaMemcpyHostToDevice, s));
      d_act = P.act.p;
    }
    launch(k_sym_gather, static_cast<unsigned>((M * M + 255) / 256), 256, 0, s, d_H, N, d_act, M, P.sub.p);
    double* const dd = P.tri.p;
    double* const ee = dd + M;
    double* const e2 = ee + M;
    double* const ww = e2 + M;
    double* const bnd = ww + M;  // 3
    int const Mi = static_cast<int>(M);
    tridiag_launch(P.sub.p, Mi, dd, ee, s);
    // Gershgorin interval and stopping width on the host (O(M) values)
    std::vector<double> hd(static_cast<std::size_t>(M)), he(static_cast<std::size_t>(M));
    FLY_CUDA(cudaMemcpyAsync(hd.data(), dd, sizeof(double) * hd.size(), cudaMemcpyDeviceToHost, s));
    FLY_CUDA(cudaMemcpyAsync(he.data(), ee, sizeof(double) * he.size(), cudaMemcpyDeviceToHost, s));
    FLY_CUDA(cudaStreamSynchronize(s));
    std::vector<double> he2(static_cast<std::size_t>(M), 0.0);
    double lo = 0, hi = 0, tnorm = 0;
    for (std::int64_t i = 0; i < M; ++i) {
      std::size_t const k = static_cast<std::size_t>(i);
      double const el = i > 0 ? std::fabs(he[k - 1]) : 0.0;
      double const er = i + 1 < M ? std::fabs(he[k]) : 0.0;
      double const a = hd[k];
      lo = i == 0 ? a - el - er : std::min(lo, a - el - er);
      hi = i == 0 ? a + el + er : std::max(hi, a + el + er);
      tnorm = std::max(tnorm, std::fabs(a) + el + er);
      if (i + 1 < M) he2[k] = he[k] * he[k];
    }
    double const pad = 2 * DBL_EPSILON * std::max(tnorm, DBL_MIN) * static_cast<double>(M) + DBL_MIN;
    double const hb[3] = {lo - pad, hi + pad, 2 * DBL_EPSILON * tnorm};
    FLY_CUDA(cudaMemcpyAsync(e2, he2.data(), sizeof(double) * he2.size(), cudaMemcpyHostToDevice, s));
    FLY_CUDA(cudaMemcpyAsync(bnd, hb, sizeof hb, cudaMemcpyHostToDevice, s));
    // one warp per block: the warps spread over every SM (binary64 throughput is per SM)
    launch(k_bisect, static_cast<unsigned>(M), 32, 0, s, static_cast<double const*>(dd), static_cast<double const*>(e2), Mi,
           static_cast<double const*>(bnd), ww);
    FLY_CUDA(cudaMemcpyAsync(h_eig, ww, sizeof(double) * static_cast<std::size_t>(M), cudaMemcpyDeviceToHost, s));
    FLY_CUDA(cudaStreamSynchronize(s));
  }

}  // namespace flygpu
