// eigen.cu -- eigenvalues of a dense symmetric binary64 matrix on the device (the prefactor step's
// Hessian::eigenvalues, system/hessian.hpp:86-93, which the reference hands to Eigen's
// SelfAdjointEigenSolver: Householder tridiagonalisation, then the tridiagonal's eigenvalues).
//
// Stage 1: Householder reduction to tridiagonal form by one thread-block cluster. CTA c of C owns the
// rows i with i mod C == c. Step k, for the trailing block below row k:
//   the reflector from row k: alpha = -sign(x0) |x| for x = A[k, k+1:], u = x - alpha e1,
//   tau = 1 / (alpha^2 - alpha x0), so H = I - tau u u^T maps x to alpha e1;
//   owned rows: p_i = tau sum_j A[i, j] u_j, and their share of u^T p;      cluster barrier;
//   K = tau / 2 sum (u^T p), w = p - K u;  owned rows: A[i, j] -= u_i w_j + w_i u_j;   cluster barrier.
// d_k = A[k, k], e_k = alpha. k_tridiag_push, when every CTA's rows fit in its shared memory (8 CTAs
// for M up to ~460, 16 up to ~640): the producers write into every CTA's shared memory before each
// barrier (the p_i and the warps' shares before the first; the owner of row k + 1 updates that row
// first, forms step k + 1's reflector from it and pushes u and tau before the second), so every step
// starts with its inputs local. k_tridiag_global, for larger M: the rows stay in the global matrix and
// each step reads row k, the p values and the shares across the cluster. Every CTA runs the same loop
// with the same trip count and no early exit, so every barrier is reached by all of them (hardware
// cluster barriers, not spin loops).
// GB300 issues binary64 at about 1/64 of the binary32 rate (1.6 lanes a clock per SM) and a dependent
// binary64 operation takes ~67 cycles, so the O(M^3) work (the rows, u, w, p and every dot product) is
// float-float arithmetic on the binary32 units (~48 significant bits, far inside the eigenvalues'
// 1e-10-of-the-spectral-radius tolerance), and so are the per-step scalars. The inner loops keep
// products as unnormalised pairs and renormalise once per element (the update) or once per row (the
// dot products).
// Stage 2, k_tri_prep then k_bisect: the tridiagonal's eigenvalues by Sturm-sequence multisection, one
// warp per eigenvalue index j: the 32 lanes count the eigenvalues below 32 points of the current
// interval (sign changes of the leading principal minors of T - x I, a division-free three-term
// recurrence), and the interval shrinks to the sub-interval holding eigenvalue j: in binary32 while it is
// wide, then, widened by the binary32 counts' reach, in float-float until it is within 4 ulp of its
// endpoints or of 2 eps |T|. Ascending order comes from j.

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

    // The same arithmetic with fewer renormalisations, for the tridiagonalisation's inner loops. A product
    // a b as the unnormalised pair p + e (exact but for a.lo b.lo), TwoSum, a dot-product step that keeps
    // its accumulator unnormalised, and the row update v - (a b + c d).
    __device__ inline void ff_prod(ff a, ff b, float& p, float& e) {
      p = __fmul_rn(a.hi, b.hi);
      e = fmaf(a.hi, b.lo, fmaf(a.lo, b.hi, fmaf(a.hi, b.hi, -p)));
    }
    __device__ inline void two_sum(float a, float b, float& s, float& err) {
      s = __fadd_rn(a, b);
      float const bb = __fsub_rn(s, a);
      err = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
    }
    __device__ inline void ff_dot_step(ff& acc, ff a, ff b) {  // acc += a b, acc.lo left unnormalised
      float p, e, s, err;
      ff_prod(a, b, p, e);
      two_sum(acc.hi, p, s, err);
      acc.hi = s;
      acc.lo = __fadd_rn(acc.lo, __fadd_rn(e, err));
    }
    __device__ inline ff ff_norm(ff a) {  // an unnormalised pair as a float-float value
      float s, err;
      two_sum(a.hi, a.lo, s, err);
      return {s, err};
    }
    __device__ inline ff ff_sub_dot2(ff v, ff a, ff b, ff c, ff d) {  // v - (a b + c d)
      float p1, e1, p2, e2, s, err, s2, err2;
      ff_prod(a, b, p1, e1);
      ff_prod(c, d, p2, e2);
      two_sum(p1, p2, s, err);
      float const t = __fadd_rn(__fadd_rn(e1, e2), err);
      two_sum(v.hi, -s, s2, err2);
      return quick_two_sum(s2, __fadd_rn(__fsub_rn(v.lo, t), err2));
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

    // A float-float element of the global matrix, read and written through L2 (ld.global.cg / st.global.cg:
    // other CTAs of the cluster write these rows between the barriers).
    __device__ inline ff ld(ff const* p) {
      float2 const v = __ldcg(reinterpret_cast<float2 const*>(p));
      return {v.x, v.y};
    }
    __device__ inline void st(ff* p, ff v) { __stcg(reinterpret_cast<float2*>(p), make_float2(v.hi, v.lo)); }

    // Householder tridiagonalisation of the M x M symmetric A (binary64, full storage) with the rows in
    // the global matrix: A is first converted in place to float-float and then overwritten. d: M, e: M
    // (e[M-1] unused). Launched as one cluster of C CTAs; CTA c owns the rows i with i mod C == c. Row k
    // is read from the matrix, the p values and the CTAs' shares of u^T p across the cluster through
    // distributed shared memory. The matrix, u, w, p and every dot product are float-float, and so are
    // the per-step scalars |x|, alpha and tau (binary32 seeds refined by one float-float Newton step).
    __global__ void __launch_bounds__(TT) k_tridiag_global(double* __restrict__ A, int M, double* __restrict__ d,
                                                          double* __restrict__ e) {
      cg::cluster_group cl = cg::this_cluster();
      int const C = static_cast<int>(cl.num_blocks());
      int const c = static_cast<int>(cl.block_rank());
      extern __shared__ ff sm[];
      ff* u = sm;                                                 // M
      ff* w = u + M;                                              // M
      ff* pl = w + M;                                             // M: p_i of the owned rows, at index i
      ff* share = pl + M;                                         // 1
      ff* red = share + 1;                                        // TW + 1
      int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      ff* const Aff = reinterpret_cast<ff*>(A);  // the rows, converted in place
      for (int r = warp; r * C + c < M; r += TW)
        for (int j = lane; j < M; j += 32) {
          std::int64_t const g = static_cast<std::int64_t>(r * C + c) * M + j;
          st(Aff + g, ff_of(__ldcg(A + g)));
        }
      cl.sync();
      for (int k = 0; k + 2 < M; ++k) {
        int const b = k + 1, m = M - b;
        ff const* rk = Aff + static_cast<std::int64_t>(k) * M;
        ff s2 = {0.f, 0.f};
        for (int j = threadIdx.x; j < m; j += TT) {
          ff const x = ld(rk + b + j);
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
          d[k] = ff_dbl(ld(rk + k));
          e[k] = ff_dbl(reflect ? alpha : x0);
        }
        __syncthreads();
        // p_i = tau (A u)_i over owned rows, and the share of u^T p. Each lane keeps four independent
        // partial sums, so a row's dependent chain is a quarter of its length.
        ff sh = {0.f, 0.f};
        for (int r = warp; r * C + c < M; r += TW) {
          int const i = r * C + c;
          if (i < b) continue;
          ff const* ri = (Aff + static_cast<std::int64_t>(i) * M) + b;
          ff acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
          int j = lane;
          for (; j + 96 < m; j += 128) {
            ff v[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) v[t] = ld(ri + j + 32 * t);
#pragma unroll
            for (int t = 0; t < 4; ++t) ff_dot_step(acc[t], v[t], u[j + 32 * t]);
          }
          for (; j < m; j += 32) ff_dot_step(acc[0], ld(ri + j), u[j]);
          ff a = ff_add(ff_add(ff_norm(acc[0]), ff_norm(acc[1])), ff_add(ff_norm(acc[2]), ff_norm(acc[3])));
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
          ff* ri = (Aff + static_cast<std::int64_t>(i) * M) + b;
          ff const ui = u[i - b], wi = w[i - b];
          // A_ij - (u_i w_j + w_i u_j)
          int j = lane;
          for (; j + 96 < m; j += 128) {
            ff v[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) v[t] = ld(ri + j + 32 * t);
#pragma unroll
            for (int t = 0; t < 4; ++t) st(ri + j + 32 * t, ff_sub_dot2(v[t], ui, w[j + 32 * t], wi, u[j + 32 * t]));
          }
          for (; j < m; j += 32) st(ri + j, ff_sub_dot2(ld(ri + j), ui, w[j], wi, u[j]));
        }
        cl.sync();
      }
      if (c == 0 && threadIdx.x == 0) {
        auto at = [&](int i, int j) {
          return ff_dbl(ld(Aff + static_cast<std::int64_t>(i) * M + j));
        };
        if (M >= 2) {
          d[M - 2] = at(M - 2, M - 2);
          e[M - 2] = at(M - 1, M - 2);
        }
        d[M - 1] = at(M - 1, M - 1);
      }
      cl.sync();  // no CTA leaves while another may still read its shared memory
    }

    // ------------------------------------------------------------------ rows in shared memory, pushed
    // The form used when every CTA's rows fit in its shared memory. Instead of reading row k, the p values
    // and the shares across the cluster after each barrier, the producers write them into every CTA's
    // shared memory before it: each warp pushes the p_i of its rows and its share of u^T p before the
    // first barrier, and the owner of row k + 1 updates that row first, forms step k + 1's reflector u and
    // tau from it with one warp, and pushes them (double-buffered by step parity) before the second. Every
    // step then starts with u and tau local, and K and w need no remote reads. Values that several CTAs
    // use (p_i, the shares, K) are formed by one lane and broadcast, so every CTA applies the same update.
    //
    // Shared memory (8-byte elements): rows R x M | u of even and odd steps 2 M | w M | p M |
    // shares C * TW | tau of even and odd steps 2.

    std::size_t tridiag_push_smem(int M, int C) {
      std::size_t const R = static_cast<std::size_t>((M + C - 1) / C);
      return (R * static_cast<std::size_t>(M) + 5 * static_cast<std::size_t>(M) + static_cast<std::size_t>(C) * TW + 2) *
             sizeof(double);
    }

    // Sum over a warp of v, formed in lane 0's order and broadcast, so every lane (and every warp that
    // sums the same values) holds the same bits.
    __device__ inline ff warp_sum_bcast(ff v) {
      for (int o = 16; o > 0; o >>= 1) v = ff_add(v, ff_shfl_down(v, o));
      return {__shfl_sync(0xffffffffu, v.hi, 0), __shfl_sync(0xffffffffu, v.lo, 0)};
    }

    // The reflector's scalars from s2 = |x|^2 and x0 (every lane of a warp, the same values): alpha, tau
    // and whether the column needs a reflection. The same operations as the cluster-wide form.
    struct Refl {
      ff alpha, tau;
      bool reflect;
    };
    __device__ inline Refl reflector_scalars(ff s2, ff x0) {
      float const sq = sqrtf(s2.hi);
      ff nrm = {0.f, 0.f};
      if (sq > 0.f) {
        ff const r = ff_add(s2, ff_neg(ff_mul(ff{sq, 0.f}, ff{sq, 0.f})));
        nrm = quick_two_sum(sq, __fdiv_rn(r.hi, 2.f * sq));
      }
      Refl o;
      o.alpha = x0.hi > 0.f ? ff_neg(nrm) : nrm;
      ff const den = ff_add(ff_mul(o.alpha, o.alpha), ff_neg(ff_mul(o.alpha, x0)));
      o.reflect = den.hi > 0.f && ff_add(s2, ff_neg(ff_mul(x0, x0))).hi > 0.f;
      o.tau = {0.f, 0.f};
      if (o.reflect) {
        float const r0 = __frcp_rn(den.hi);
        ff const e1 = ff_add(ff{1.f, 0.f}, ff_neg(ff_mul(den, ff{r0, 0.f})));
        o.tau = quick_two_sum(r0, __fmul_rn(r0, e1.hi));
      }
      return o;
    }

    // Lane 0 of the owner's warp: u[0], tau, d[s] and e[s] of step s (diag = A[s, s], x0 = A[s, s+1]).
    __device__ inline void finish_reflector(Refl const& q, ff x0, ff diag, int s, ff* u, ff* tau, double* d, double* e) {
      u[0] = q.reflect ? ff_add(x0, ff_neg(q.alpha)) : ff{0.f, 0.f};
      *tau = q.tau;
      d[s] = ff_dbl(diag);
      e[s] = ff_dbl(q.reflect ? q.alpha : x0);
    }

    // One warp of the owner of row s: the reflector of step s from x = A[s, s+1:] (row points at row s),
    // u into u (M - s - 1 values) and tau into *tau; d[s] = A[s, s] and e[s] = alpha (x0 when the column
    // needs no reflection).
    __device__ void form_reflector(ff const* row, int s, int M, ff* u, ff* tau, double* d, double* e) {
      int const lane = threadIdx.x & 31;
      int const b = s + 1, m = M - b;
      ff s2 = {0.f, 0.f};
      for (int j = lane; j < m; j += 32) {
        ff const x = row[b + j];
        u[j] = x;
        s2 = ff_add(s2, ff_mul(x, x));
      }
      s2 = warp_sum_bcast(s2);
      ff const x0 = row[b];
      Refl const q = reflector_scalars(s2, x0);
      __syncwarp();
      if (lane == 0) finish_reflector(q, x0, row[s], s, u, tau, d, e);
      __syncwarp();
    }

    // The owner's warp 0 at step k (row b = k + 1, ri = row b from column b, m = M - b): updates row b and,
    // in the same pass, gathers step k + 1's x = A[b, b+1:] into un and its |x|^2; then the reflector.
    __device__ void update_and_reflect(ff* ri, ff ui, ff wi, ff const* u, ff const* w, int m, int b, ff* un,
                                       ff* tau, double* d, double* e) {
      int const lane = threadIdx.x & 31;
      ff s2 = {0.f, 0.f};
      for (int j = lane; j < m; j += 32) {
        ff const v = ff_sub_dot2(ri[j], ui, w[j], wi, u[j]);
        ri[j] = v;
        if (j >= 1) {
          un[j - 1] = v;
          s2 = ff_add(s2, ff_mul(v, v));
        }
      }
      s2 = warp_sum_bcast(s2);
      __syncwarp();
      ff const x0 = ri[1];
      Refl const q = reflector_scalars(s2, x0);
      __syncwarp();
      if (lane == 0) finish_reflector(q, x0, ri[0], b, un, tau, d, e);
      __syncwarp();
    }

    // Row update A_ij -= u_i w_j + w_i u_j over j < m (ri points at column b of row i), one warp.
    __device__ inline void update_row(ff* ri, ff ui, ff wi, ff const* u, ff const* w, int m) {
      int const lane = threadIdx.x & 31;
      int j = lane;
      for (; j + 96 < m; j += 128) {
        ff v[4];
#pragma unroll
        for (int t = 0; t < 4; ++t) v[t] = ri[j + 32 * t];
#pragma unroll
        for (int t = 0; t < 4; ++t) ri[j + 32 * t] = ff_sub_dot2(v[t], ui, w[j + 32 * t], wi, u[j + 32 * t]);
      }
      for (; j < m; j += 32) ri[j] = ff_sub_dot2(ri[j], ui, w[j], wi, u[j]);
    }

    // One warp of the owner copies step s's u (m values) and tau from its shared memory into every other
    // CTA's.
    __device__ inline void push_reflector(cg::cluster_group& cl, ff const* u, ff const* tau, int m) {
      int const C = static_cast<int>(cl.num_blocks()), c = static_cast<int>(cl.block_rank());
      int const lane = threadIdx.x & 31;
      for (int dst = 0; dst < C; ++dst) {
        if (dst == c) continue;
        ff* const ru = cl.map_shared_rank(const_cast<ff*>(u), dst);
        for (int j = lane; j < m; j += 32) ru[j] = u[j];
      }
      if (lane < C && lane != c) *cl.map_shared_rank(const_cast<ff*>(tau), lane) = *tau;
    }

    // The whole owner CTA copies step s's u (m values) and tau into every other CTA's shared memory.
    __device__ inline void push_reflector_cta(cg::cluster_group& cl, ff const* u, ff const* tau, int m) {
      int const C = static_cast<int>(cl.num_blocks()), c = static_cast<int>(cl.block_rank());
      for (int dst = 0; dst < C; ++dst) {
        if (dst == c) continue;
        ff* const ru = cl.map_shared_rank(const_cast<ff*>(u), dst);
        for (int j = threadIdx.x; j < m; j += TT) ru[j] = u[j];
      }
      if (static_cast<int>(threadIdx.x) < C && static_cast<int>(threadIdx.x) != c)
        *cl.map_shared_rank(const_cast<ff*>(tau), threadIdx.x) = *tau;
    }

    __global__ void __launch_bounds__(TT) k_tridiag_push(double const* __restrict__ A, int M, double* __restrict__ d,
                                                        double* __restrict__ e) {
      cg::cluster_group cl = cg::this_cluster();
      int const C = static_cast<int>(cl.num_blocks());
      int const c = static_cast<int>(cl.block_rank());
      int const R = (M + C - 1) / C;
      extern __shared__ ff sm[];
      ff* const rows = sm;                                        // R x M: row r * C + c at rows + r M
      ff* const ub = rows + static_cast<std::int64_t>(R) * M;     // 2 M
      ff* const w = ub + 2 * M;                                   // M
      ff* const pa = w + M;                                       // M: p_i of every row
      ff* const shs = pa + M;                                     // C * TW
      ff* const tb = shs + C * TW;                                // 2
      int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      for (int r = warp; r * C + c < M; r += TW)
        for (int j = lane; j < M; j += 32)
          rows[static_cast<std::int64_t>(r) * M + j] = ff_of(__ldcg(A + static_cast<std::int64_t>(r * C + c) * M + j));
      cl.sync();  // every CTA runs, so its shared memory may be written
      if (M >= 3 && c == 0 && warp == 0) {  // step 0's reflector, from row 0
        form_reflector(rows, 0, M, ub, tb, d, e);
        push_reflector(cl, ub, tb, M - 1);
      }
      cl.sync();
      for (int k = 0; k + 2 < M; ++k) {
        int const b = k + 1, m = M - b, cb = k & 1;
        ff const* const u = ub + cb * M;
        ff const tau = tb[cb];
        int const r0 = (b - c + C - 1) / C;  // the first owned row at or below row b
        // p_i = tau (A u)_i of the owned rows, pushed to every CTA, and the warp's share of u^T p
        ff sh = {0.f, 0.f};
        for (int r = r0 + warp; r < R && r * C + c < M; r += TW) {
          int const i = r * C + c;
          ff const* ri = rows + static_cast<std::int64_t>(r) * M + b;
          ff acc[4] = {{0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}, {0.f, 0.f}};
          int j = lane;
          for (; j + 96 < m; j += 128) {
            ff v[4];
#pragma unroll
            for (int t = 0; t < 4; ++t) v[t] = ri[j + 32 * t];
#pragma unroll
            for (int t = 0; t < 4; ++t) ff_dot_step(acc[t], v[t], u[j + 32 * t]);
          }
          for (; j < m; j += 32) ff_dot_step(acc[0], ri[j], u[j]);
          ff const a =
            warp_sum_bcast(ff_add(ff_add(ff_norm(acc[0]), ff_norm(acc[1])), ff_add(ff_norm(acc[2]), ff_norm(acc[3]))));
          ff const pi = ff_mul(tau, a);
          if (lane < C) *cl.map_shared_rank(pa + i, lane) = pi;
          sh = ff_add(sh, ff_mul(u[i - b], pi));
        }
        if (lane < C) cl.map_shared_rank(shs, lane)[c * TW + warp] = sh;
        cl.sync();
        // K = tau / 2 sum of every warp's share: the same order in every warp of every CTA (each lane
        // adds its shares pairwise: at most 8, for 16 CTAs of 16 warps; missing ones are zeros)
        ff t[8];
#pragma unroll
        for (int q = 0; q < 8; ++q) t[q] = lane + 32 * q < C * TW ? shs[lane + 32 * q] : ff{0.f, 0.f};
        if (C * TW > 128) {
#pragma unroll
          for (int q = 0; q < 4; ++q) t[q] = ff_add(t[q], t[q + 4]);
        }
        t[0] = ff_add(ff_add(t[0], t[2]), ff_add(t[1], t[3]));
        ff const K = ff_mul(ff_mul(tau, warp_sum_bcast(t[0])), ff{0.5f, 0.f});
        for (int j = threadIdx.x; j < m; j += TT) w[j] = ff_add(pa[b + j], ff_neg(ff_mul(K, u[j])));
        __syncthreads();
        bool const next = k + 3 < M;  // a step k + 1 follows
        if (c == b % C) {
          // this CTA owns row b: warp 0 updates it and forms step k + 1's reflector from it while the
          // other warps update the remaining rows; then the whole CTA pushes the reflector
          if (warp == 0) {
            ff* const rb = rows + static_cast<std::int64_t>(r0) * M + b;
            if (next) update_and_reflect(rb, u[0], w[0], u, w, m, b, ub + (cb ^ 1) * M, tb + (cb ^ 1), d, e);
            else update_row(rb, u[0], w[0], u, w, m);
          } else {
            for (int r = r0 + warp; r < R && r * C + c < M; r += TW - 1) {
              int const i = r * C + c;
              update_row(rows + static_cast<std::int64_t>(r) * M + b, u[i - b], w[i - b], u, w, m);
            }
          }
          __syncthreads();
          if (next) push_reflector_cta(cl, ub + (cb ^ 1) * M, tb + (cb ^ 1), m - 1);
        } else {
          for (int r = r0 + warp; r < R && r * C + c < M; r += TW) {
            int const i = r * C + c;
            update_row(rows + static_cast<std::int64_t>(r) * M + b, u[i - b], w[i - b], u, w, m);
          }
        }
        cl.sync();
      }
      if (c == 0 && threadIdx.x == 0) {
        auto at = [&](int i, int j) { return ff_dbl(cl.map_shared_rank(rows, i % C)[static_cast<std::int64_t>(i / C) * M + j]); };
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
        // (d_i - x) p - e_{i-1}^2 pm: both products as unnormalised pairs, one TwoSum of their leading
        // parts, one renormalisation (the product with pm is off the recurrence's dependent chain)
        float p1, e1, p2, e2x, s, err;
        ff_prod(ff_add(d[i], nx), p, p1, e1);
        ff_prod(e2[i - 1], pm, p2, e2x);
        two_sum(p1, -p2, s, err);
        ff pn = quick_two_sum(s, __fadd_rn(__fsub_rn(e1, e2x), err));
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

    // The same count in binary32 (the high parts of d and e^2). It is the exact count of a tridiagonal
    // within about 8 eps32 |T| of T (each step's rounding perturbs d_i - x and e_{i-1}^2 relatively by a
    // few eps32, and the rounding of the data and of x adds eps32 |T|): so a count of more than j at x
    // puts eigenvalue j below x + delta, and a count of at most j puts it at or above x - delta, for the
    // delta that k_tri_prep supplies (32 eps32 |T|).
    __device__ int sturm_count32(ff const* __restrict__ d, ff const* __restrict__ e2, int M, float x) {
      float pm = 1.f;
      float p = __fsub_rn(d[0].hi, x);
      if (p == 0.f) p = -0x1p-40f;
      int cnt = p < 0.f;
      for (int i = 1; i < M; ++i) {
        float pn = fmaf(__fsub_rn(d[i].hi, x), p, -__fmul_rn(e2[i - 1].hi, pm));
        if (pn == 0.f) pn = -p * 0x1p-40f;
        cnt += (pn < 0.f) != (p < 0.f);
        pm = p;
        p = pn;
        float const ap = fabsf(p);
        if (ap > 0x1p60f) {
          p *= 0x1p-64f;
          pm *= 0x1p-64f;
        } else if (ap < 0x1p-60f && fabsf(pm) < 0x1p-60f) {
          p *= 0x1p64f;
          pm *= 0x1p64f;
        }
      }
      return cnt;
    }

    // One warp per eigenvalue index j; bounds = {lo, hi, tol, flag, delta} (binary64). Each round the 32
    // lanes count the eigenvalues below 32 points that split the interval into 33 equal parts, and the
    // interval becomes the part holding eigenvalue j. The rounds run in binary32 (a recurrence step a
    // quarter as long) while the interval is wider than 16 delta; the interval is then widened by delta
    // on both sides, which keeps eigenvalue j inside it, and the float-float rounds finish it.
    __global__ void __launch_bounds__(32) k_bisect(ff const* __restrict__ d, ff const* __restrict__ e2, int M,
                                                  double const* __restrict__ bounds, double* __restrict__ eig) {
      int const lane = threadIdx.x & 31;
      int const j = blockIdx.x;
      double lo = bounds[0], hi = bounds[1];
      double const tol = bounds[2], delta = bounds[4];
      bool fast = true;
      for (int it = 0; it < 96; ++it) {
        double const width = hi - lo;
        if (fast && !(width > 16 * delta)) {
          fast = false;
          lo -= delta;
          hi += delta;
          continue;
        }
        if (!fast && width <= fmax(tol, 4 * DBL_EPSILON * fmax(fabs(lo), fabs(hi)))) break;
        double const step = width * (1.0 / 33.0);
        double const x = lo + step * static_cast<double>(lane + 1);
        int const cnt = fast ? sturm_count32(d, e2, M, __double2float_rn(x)) : sturm_count(d, e2, M, ff_of(x));
        unsigned const above = __ballot_sync(0xffffffffu, cnt > j);
        int const f = above ? __ffs(above) - 1 : 32;  // the first point with more than j below it
        // the same expression as x for points f - 1 and f
        double const xf = lo + step * static_cast<double>(f + 1);
        double const xp = lo + step * static_cast<double>(f);
        if (f == 32) {
          lo = xp;
        } else {
          hi = xf;
          if (f > 0) lo = xp;
        }
      }
      if (lane == 0) eig[j] = 0.5 * (lo + hi);
    }

    // The multisection's inputs from the tridiagonal (d, e; one CTA): d and e^2 as float-float, and
    // bounds = {lo, hi, tol, flag, delta}: the Gershgorin interval of T padded by 2 eps |T| M, the stopping
    // width 2 eps |T|, flag = 1 when |T| >= 2^30 (the recurrences' products e^2 p stay inside binary32's range
    // below that: p is kept within 2^-60 .. 2^60), and delta = 32 eps32 |T|.
    constexpr int PREP_T = 1024;
    __global__ void __launch_bounds__(PREP_T) k_tri_prep(double const* __restrict__ d, double const* __restrict__ e, int M,
                                                        ff* __restrict__ dff, ff* __restrict__ e2ff,
                                                        double* __restrict__ bounds) {
      __shared__ double red[3][PREP_T / 32];
      int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      double lo = INFINITY, hi = -INFINITY, tn = 0;
      for (int i = threadIdx.x; i < M; i += PREP_T) {
        double const el = i > 0 ? fabs(e[i - 1]) : 0.0;
        double const er = i + 1 < M ? fabs(e[i]) : 0.0;
        double const a = d[i];
        lo = fmin(lo, a - el - er);
        hi = fmax(hi, a + el + er);
        tn = fmax(tn, fabs(a) + el + er);
        dff[i] = ff_of(a);
        e2ff[i] = i + 1 < M ? ff_of(e[i] * e[i]) : ff{0.f, 0.f};
      }
      for (int o = 16; o > 0; o >>= 1) {
        lo = fmin(lo, __shfl_xor_sync(0xffffffffu, lo, o));
        hi = fmax(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        tn = fmax(tn, __shfl_xor_sync(0xffffffffu, tn, o));
      }
      if (lane == 0) {
        red[0][warp] = lo;
        red[1][warp] = hi;
        red[2][warp] = tn;
      }
      __syncthreads();
      if (threadIdx.x == 0) {
        for (int w = 1; w < PREP_T / 32; ++w) {
          lo = fmin(lo, red[0][w]);
          hi = fmax(hi, red[1][w]);
          tn = fmax(tn, red[2][w]);
        }
        double const pad = 2 * DBL_EPSILON * fmax(tn, DBL_MIN) * static_cast<double>(M) + DBL_MIN;
        bounds[0] = lo - pad;
        bounds[1] = hi + pad;
        bounds[2] = 2 * DBL_EPSILON * tn;
        bounds[3] = tn < 0x1p30 ? 0.0 : 1.0;
        bounds[4] = 32 * 0x1p-24 * tn;  // the binary32 counts' reach (k_bisect)
      }
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

    std::size_t tridiag_global_smem(int M) {  // u, w, p (M each), the share and TW + 1 reduction slots
      return (3 * static_cast<std::size_t>(M) + 1 + TW + 1) * sizeof(double);  // 8-byte elements
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

    // Whether a cluster of C CTAs of kernel k with smem bytes each can run on this device.
    template <class K>
    bool cluster_fits(K k, int C, std::size_t smem) {
      if (smem > static_cast<std::size_t>(TRIDIAG_SMEM_MAX)) return false;
      cudaLaunchAttribute at{};
      cudaLaunchConfig_t const cfg = tridiag_config(C, smem, at, nullptr);
      int n = 0;
      bool const ok = cudaOccupancyMaxActiveClusters(&n, k, &cfg) == cudaSuccess && n > 0;
      cudaGetLastError();
      return ok;
    }

    // Launches the tridiagonalisation of the M x M matrix A (global) on stream s: with the rows in shared
    // memory (k_tridiag_push) on the first cluster of 8, 16, 4, ... CTAs that holds them, else in the
    // global matrix on the largest cluster the device can hold. The kernels' shared-memory limits are set to the same constant on every
    // call, so concurrent callers agree.
    void tridiag_launch(double* A, int M, double* d, double* e, cudaStream_t s) {
      FLY_CUDA(cudaFuncSetAttribute(k_tridiag_push, cudaFuncAttributeMaxDynamicSharedMemorySize, TRIDIAG_SMEM_MAX));
      FLY_CUDA(cudaFuncSetAttribute(k_tridiag_push, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      FLY_CUDA(cudaFuncSetAttribute(k_tridiag_global, cudaFuncAttributeMaxDynamicSharedMemorySize, TRIDIAG_SMEM_MAX));
      FLY_CUDA(cudaFuncSetAttribute(k_tridiag_global, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
      for (int C : {8, 16, 4, 2, 1}) {
        std::size_t const sp = tridiag_push_smem(M, C);
        if (!cluster_fits(k_tridiag_push, C, sp)) continue;
        cudaLaunchAttribute at{};
        cudaLaunchConfig_t const cfg = tridiag_config(C, sp, at, s);
        FLY_CUDA(cudaLaunchKernelEx(&cfg, k_tridiag_push, static_cast<double const*>(A), M, d, e));
        count_launch();
        return;
      }
      for (int C : {16, 8, 4, 2, 1}) {
        std::size_t const sg = tridiag_global_smem(M);
        if (!cluster_fits(k_tridiag_global, C, sg)) continue;
        cudaLaunchAttribute at{};
        cudaLaunchConfig_t const cfg = tridiag_config(C, sg, at, s);
        FLY_CUDA(cudaLaunchKernelEx(&cfg, k_tridiag_global, A, M, d, e));
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
    double* const bnd = ww + M;  // 5
    int const Mi = static_cast<int>(M);
    tridiag_launch(P.sub.p, Mi, dd, ee, s);
    // d and e^2 as float-float pairs, the Gershgorin interval and the stopping width, on the device
    ff* const dff = reinterpret_cast<ff*>(fb);
    launch(k_tri_prep, 1, PREP_T, 0, s, static_cast<double const*>(dd), static_cast<double const*>(ee), Mi, dff, dff + M,
           bnd);
    // one warp per block: the warps spread over every SM
    launch(k_bisect, static_cast<unsigned>(M), 32, 0, s, static_cast<ff const*>(dff), static_cast<ff const*>(dff + M), Mi,
           static_cast<double const*>(bnd), ww);
    double flag = 0;
    FLY_CUDA(cudaMemcpyAsync(h_eig, ww, sizeof(double) * static_cast<std::size_t>(M), cudaMemcpyDeviceToHost, s));
    FLY_CUDA(cudaMemcpyAsync(&flag, bnd + 3, sizeof(double), cudaMemcpyDeviceToHost, s));
    FLY_CUDA(cudaStreamSynchronize(s));
    if (flag != 0) fail(FLYGPU_INVALID_ARG, "matrix norm beyond the eigensolver's float-float range");
  }

}  // namespace flygpu
