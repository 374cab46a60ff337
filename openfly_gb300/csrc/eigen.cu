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
// GB300 issues binary64 at about 1/64 of the binary32 rate (1.6 lanes a clock per SM) and a dependent
// binary64 operation takes ~67 cycles, so the O(M^3) work (the rows, u, w, p and every dot product) is
// float-float arithmetic on the binary32 units (~48 significant bits, far inside the eigenvalues'
// 1e-10-of-the-spectral-radius tolerance), and so are the per-step scalars. Reductions run on the
// warps that hold data, and rows are walked in full groups of four plus a one-wide tail.
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

    // ------------------------------------------------------------------ float-float arithmetic
    // A value as an unevaluated sum hi + lo of two binary32 numbers (|lo| <= ulp(hi) / 2): about 48
    // significant bits, from binary32 instructions only. The error-free steps (TwoSum, the FMA split of a
    // product) use the _rn intrinsics so the compiler cannot fuse or reorder them.
    struct ff {
      float hi, lo;
    };
    __device__ inline ff ff_of(double d) {
      float const h = __double2float_rn(d);
      return {h, __double2float_rn(d - static_cast<double>(h))};
    }
    __device__ inline double ff_dbl(ff a) { return static_cast<double>(a.hi) + static_cast<double>(a.lo); }
    __device__ inline ff quick_two_sum(float a, float b) {  // |a| >= |b| or a == 0
      float const s = __fadd_rn(a, b);
      return {s, __fsub_rn(b, __fsub_rn(s, a))};
    }
    __device__ inline ff ff_add(ff a, ff b) {
      float const s = __fadd_rn(a.hi, b.hi);
      float const bb = __fsub_rn(s, a.hi);
      float const e = __fadd_rn(__fsub_rn(a.hi, __fsub_rn(s, bb)), __fsub_rn(b.hi, bb));
      return quick_two_sum(s, __fadd_rn(e, __fadd_rn(a.lo, b.lo)));
    }
    __device__ inline ff ff_mul(ff a, ff b) {
      float const p = __fmul_rn(a.hi, b.hi);
      float e = fmaf(a.hi, b.hi, -p);
      e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, e));
      return quick_two_sum(p, e);
    }
    __device__ inline ff ff_neg(ff a) { return {-a.hi, -a.lo}; }
    __device__ inline ff ff_shfl_down(ff a, int o) {
      return {__shfl_down_sync(0xffffffffu, a.hi, o), __shfl_down_sync(0xffffffffu, a.lo, o)};
    }
    __device__ inline ff ff_shfl_xor(ff a, int o) {
      return {__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
    }

    // Sum over the CTA of v, where only warps w < nw hold data: their lanes reduce with shuffles, their
    // leaders' sums are added by warp 0.
    __device__ ff cta_sum(ff v, ff* red, int nw) {
      int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      if (warp < nw) {
        for (int o = 16; o > 0; o >>= 1) v = ff_add(v, ff_shfl_down(v, o));
        if (lane == 0) red[warp] = v;
      }
      __syncthreads();
      if (warp == 0) {
        ff t = lane < nw ? red[lane] : ff{0.f, 0.f};
        for (int o = 16; o > 0; o >>= 1) t = ff_add(t, ff_shfl_down(t, o));
        if (lane == 0) red[TW] = t;
      }
      __syncthreads();
      ff const s = red[TW];
      __syncthreads();
      return s;
    }

    // The rows of the matrix a CTA owns: in its shared memory (SM) or in the global matrix, as float-float.
    template <bool SM>
    struct Rows {
      ff* base;  // SM: the CTA's rows, local row r at base + r M; else the global matrix
      int M, C;
      __device__ ff* own(int i) const {
        return SM ? base + static_cast<std::int64_t>(i / C) * M : base + static_cast<std::int64_t>(i) * M;
      }
    };

    template <bool SM>
    __device__ inline ff ld(ff const* p) {
      if constexpr (SM) {
        return *p;
      } else {
        float2 const v = __ldcg(reinterpret_cast<float2 const*>(p));
        return {v.x, v.y};
      }
    }
    template <bool SM>
    __device__ inline void st(ff* p, ff v) {
      if constexpr (SM) {
        *p = v;
      } else {
        __stcg(reinterpret_cast<float2*>(p), make_float2(v.hi, v.lo));
      }
    }

    // Householder tridiagonalisation of the M x M symmetric A (binary64, full storage; overwritten on
    // the global path, where it is first converted in place to float-float). d: M, e: M (e[M-1]
    // unused). Launched as one cluster of C CTAs; CTA c owns the rows i with i mod C == c. With SM every
    // CTA keeps its rows in shared memory (ceil(M / C) rows). Row k, the p values and the CTAs' shares
    // of u^T p are read across the cluster through distributed shared memory. The matrix, u, w, p and
    // every dot product are float-float, and so are the per-step scalars |x|, alpha and tau (binary32
    // seeds refined by one float-float Newton step).
    template <bool SM>
    __global__ void __launch_bounds__(TT) k_tridiag(double* __restrict__ A, int M, double* __restrict__ d,
                                                   double* __restrict__ e) {
      cg::cluster_group cl = cg::this_cluster();
      int const C = static_cast<int>(cl.num_blocks());
      int const c = static_cast<int>(cl.block_rank());
      int const R = (M + C - 1) / C;
      extern __shared__ ff sm[];
      ff* rows = sm;                                              // SM: R x M
      ff* u = sm + (SM ? static_cast<std::int64_t>(R) * M : 0);  // M
      ff* w = u + M;                                              // M
      ff* pl = w + M;                                             // M: p_i of the owned rows, at index i
      ff* share = pl + M;                                         // 1
      ff* red = share + 1;                                        // TW + 1
      int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      ff* const Aff = reinterpret_cast<ff*>(A);  // the global path's rows, converted in place
      Rows<SM> const own{SM ? rows : Aff, M, C};
      for (int r = warp; r * C + c < M; r += TW)
        for (int j = lane; j < M; j += 32) {
          std::int64_t const g = static_cast<std::int64_t>(r * C + c) * M + j;
          ff const v = ff_of(__ldcg(A + g));
          if (SM) {
            rows[static_cast<std::int64_t>(r) * M + j] = v;
          } else {
            st<false>(Aff + g, v);
          }
        }
      cl.sync();
      for (int k = 0; k + 2 < M; ++k) {
        int const b = k + 1, m = M - b;
        ff const* rk = SM ? cl.map_shared_rank(rows, k % C) + static_cast<std::int64_t>(k / C) * M
                          : Aff + static_cast<std::int64_t>(k) * M;
        ff s2 = {0.f, 0.f};
        for (int j = threadIdx.x; j < m; j += TT) {
          ff const x = ld<SM>(rk + b + j);
          u[j] = x;
          s2 = ff_add(s2, ff_mul(x, x));
        }
        s2 = cta_sum(s2, red, min(TW, (m + 31) / 32));
        // |x| and tau = 1 / (alpha^2 - alpha x0) from binary32 seeds with one float-float Newton step
        ff const x0 = u[0];
        float const sq = sqrtf(s2.hi);
        ff nrm = {0.f, 0.f};
        if (sq > 0.f) {
          ff const r = ff_add(s2, ff_neg(ff_mul(ff{sq, 0.f}, ff{sq, 0.f})));
          nrm = quick_two_sum(sq, __fdiv_rn(r.hi, 2.f * sq));
        }
        ff const alpha = x0.hi > 0.f ? ff_neg(nrm) : nrm;
        ff const den = ff_add(ff_mul(alpha, alpha), ff_neg(ff_mul(alpha, x0)));
        // a column that is already zero below the sub-diagonal needs no reflection (tau = 0)
        bool const reflect = den.hi > 0.f && ff_add(s2, ff_neg(ff_mul(x0, x0))).hi > 0.f;
        ff tau = {0.f, 0.f};
        if (reflect) {
          float const r0 = __frcp_rn(den.hi);
          ff const e1 = ff_add(ff{1.f, 0.f}, ff_neg(ff_mul(den, ff{r0, 0.f})));
          tau = quick_two_sum(r0, __fmul_rn(r0, e1.hi));
        }
        __syncthreads();
        if (threadIdx.x == 0) u[0] = reflect ? ff_add(x0, ff_neg(alpha)) : ff{0.f, 0.f};
        if (c == 0 && threadIdx.x == 0) {
          d[k] = ff_dbl(ld<SM>(rk + k));
          e[k] = ff_dbl(reflect ? alpha : x0);
        }
        __syncthreads();
        // p_i = tau (A u)_i over owned rows, and the share of u^T p. Each lane keeps four independent
        // partial sums, so a row's dependent chain is a quarter of its length.
        ff sh = {0.f, 0.f};
        for (int r = warp; r * C + c < M; r += TW) {
          int const i = r * C + c;
          if (i < b) continue;
          ff const* ri = own.own(i) + b;
          ff acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
          int j = lane;
          for (; j + 96 < m; j += 128) {
            ff v[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) v[t] = ld<SM>(ri + j + 32 * t);
#pragma unroll
            for (int t = 0; t < 4; ++t) acc[t] = ff_add(acc[t], ff_mul(v[t], u[j + 32 * t]));
          }
          for (; j < m; j += 32) acc[0] = ff_add(acc[0], ff_mul(ld<SM>(ri + j), u[j]));
          ff a = ff_add(ff_add(acc[0], acc[1]), ff_add(acc[2], acc[3]));
          for (int o = 16; o > 0; o >>= 1) a = ff_add(a, ff_shfl_down(a, o));
          if (lane == 0) {
            ff const pi = ff_mul(tau, a);
            pl[i] = pi;
            sh = ff_add(sh, ff_mul(u[i - b], pi));
          }
        }
        // the share: one value per warp leader, summed by warp 0
        if (lane == 0) red[warp] = sh;
        __syncthreads();
        if (warp == 0) {
          ff t = lane < TW ? red[lane] : ff{0.f, 0.f};
          for (int o = 16; o > 0; o >>= 1) t = ff_add(t, ff_shfl_down(t, o));
          if (lane == 0) *share = t;
        }
        cl.sync();
        // K = tau / 2 sum of the CTAs' shares: a shuffle tree in warp 0, broadcast through shared memory
        if (warp == 0) {
          ff t = lane < C ? *cl.map_shared_rank(share, lane) : ff{0.f, 0.f};
          for (int o = 16; o > 0; o >>= 1) t = ff_add(t, ff_shfl_xor(t, o));
          if (lane == 0) red[TW] = ff_mul(ff_mul(tau, t), ff{0.5f, 0.f});
        }
        __syncthreads();
        ff const K = red[TW];
        for (int j = threadIdx.x; j < m; j += TT)
          w[j] = ff_add(cl.map_shared_rank(pl, (b + j) % C)[b + j], ff_neg(ff_mul(K, u[j])));
        __syncthreads();
        for (int r = warp; r * C + c < M; r += TW) {
          int const i = r * C + c;
          if (i < b) continue;
          ff* ri = own.own(i) + b;
          ff const ui = u[i - b], wi = w[i - b];
          // A_ij - (u_i w_j + w_i u_j)
          int j = lane;
          for (; j + 96 < m; j += 128) {
            ff v[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) v[t] = ld<SM>(ri + j + 32 * t);
#pragma unroll
            for (int t = 0; t < 4; ++t)
              st<SM>(ri + j + 32 * t, ff_add(v[t], ff_neg(ff_add(ff_mul(ui, w[j + 32 * t]), ff_mul(wi, u[j + 32 * t])))));
          }
          for (; j < m; j += 32) st<SM>(ri + j, ff_add(ld<SM>(ri + j), ff_neg(ff_add(ff_mul(ui, w[j]), ff_mul(wi, u[j])))));
        }
        cl.sync();
      }
      if (c == 0 && threadIdx.x == 0) {
        auto at = [&](int i, int j) {
          return ff_dbl(SM ? cl.map_shared_rank(rows, i % C)[static_cast<std::int64_t>(i / C) * M + j]
                           : ld<false>(Aff + static_cast<std::int64_t>(i) * M + j));
        };
        if (M >= 2) {
          d[M - 2] = at(M - 2, M - 2);
          e[M - 2] = at(M - 1, M - 2);
        }
        d[M - 1] = at(M - 1, M - 1);
      }
      cl.sync();  // no CTA leaves while another may still read its shared memory
    }

    // Number of eigenvalues of the tridiagonal (d, e2 = e^2, as float-float) below x: the sign changes
    // of the sequence 1, p_0, p_1, ... of leading principal minors of T - x I,
    // p_i = (d_i - x) p_{i-1} - e_{i-1}^2 p_{i-2} (the Sturm sequence), in float-float arithmetic on the
    // binary32 units and without divisions. A zero minor takes the sign opposite to the one before it.
    // After every step the last two minors are rescaled by 2^-64 (2^64) when they leave [2^-60, 2^60]:
    // power-of-two scaling is exact and keeps every sign, and binary32's exponent range is small.
    __device__ int sturm_count(ff const* __restrict__ d, ff const* __restrict__ e2, int M, ff x) {
      ff const nx = ff_neg(x);
      ff pm = {1.f, 0.f};
      ff p = ff_add(d[0], nx);
      if (p.hi == 0.f) p = {-0x1p-40f, 0.f};
      int cnt = p.hi < 0.f;
      for (int i = 1; i < M; ++i) {
        ff pn = ff_add(ff_mul(ff_add(d[i], nx), p), ff_neg(ff_mul(e2[i - 1], pm)));
        if (pn.hi == 0.f) pn = {-p.hi * 0x1p-40f, 0.f};
        cnt += (pn.hi < 0.f) != (p.hi < 0.f);
        pm = p;
        p = pn;
        float const ap = fabsf(p.hi);
        if (ap > 0x1p60f) {
          p = {p.hi * 0x1p-64f, p.lo * 0x1p-64f};
          pm = {pm.hi * 0x1p-64f, pm.lo * 0x1p-64f};
        } else if (ap < 0x1p-60f && fabsf(pm.hi) < 0x1p-60f) {
          p = {p.hi * 0x1p64f, p.lo * 0x1p64f};
          pm = {pm.hi * 0x1p64f, pm.lo * 0x1p64f};
        }
      }
      return cnt;
    }

    // One warp per eigenvalue index; bounds = {lo, hi, tol} (binary64).
    __global__ void k_bisect(ff const* __restrict__ d, ff const* __restrict__ e2, int M,
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
        int const cnt = sturm_count(d, e2, M, ff_of(x));
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
      return (R * static_cast<std::size_t>(M) + 3 * static_cast<std::size_t>(M) + 1 + TW + 1) * sizeof(double);  // 8-byte elements
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
    P.tri.reserve(5 * static_cast<std::size_t>(M) + 8);
    int const* d_act = nullptr;
    if (!act.empty()) {
      P.act.reserve(act.size());
      FLY_CUDA(cudaMemcpyAsync(P.act.p, act.data(), sizeof(int) * act.size(), cudaMemcpyHostToDevice, s));
      d_act = P.act.p;
    }
    launch(k_sym_gather, static_cast<unsigned>((M * M + 255) / 256), 256, 0, s, d_H, N, d_act, M, P.sub.p);
    double* const dd = P.tri.p;
    double* const ee = dd + M;
    double* const fb = ee + M;   // 2 M: d and e^2 as float-float (4 M floats)
    double* const ww = fb + 2 * M;
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
    if (!(tnorm < 1e18)) fail(FLYGPU_INVALID_ARG, "matrix norm beyond the eigensolver's float-float range");
    double const pad = 2 * DBL_EPSILON * std::max(tnorm, DBL_MIN) * static_cast<double>(M) + DBL_MIN;
    double const hb[3] = {lo - pad, hi + pad, 2 * DBL_EPSILON * tnorm};
    // d and e^2 as float-float pairs (hi, lo) for the multisection
    std::vector<float> hff(4 * static_cast<std::size_t>(M));
    for (std::int64_t i = 0; i < M; ++i) {
      std::size_t const k = static_cast<std::size_t>(i);
      float const dh = static_cast<float>(hd[k]), eh = static_cast<float>(he2[k]);
      hff[2 * k] = dh;
      hff[2 * k + 1] = static_cast<float>(hd[k] - static_cast<double>(dh));
      hff[2 * static_cast<std::size_t>(M) + 2 * k] = eh;
      hff[2 * static_cast<std::size_t>(M) + 2 * k + 1] = static_cast<float>(he2[k] - static_cast<double>(eh));
    }
    ff* const dff = reinterpret_cast<ff*>(fb);
    FLY_CUDA(cudaMemcpyAsync(dff, hff.data(), sizeof(float) * hff.size(), cudaMemcpyHostToDevice, s));
    FLY_CUDA(cudaMemcpyAsync(bnd, hb, sizeof hb, cudaMemcpyHostToDevice, s));
    // one warp per block: the warps spread over every SM
    launch(k_bisect, static_cast<unsigned>(M), 32, 0, s, static_cast<ff const*>(dff), static_cast<ff const*>(dff + M), Mi,
           static_cast<double const*>(bnd), ww);
    FLY_CUDA(cudaMemcpyAsync(h_eig, ww, sizeof(double) * static_cast<std::size_t>(M), cudaMemcpyDeviceToHost, s));
    FLY_CUDA(cudaStreamSynchronize(s));
  }

}  // namespace flygpu
