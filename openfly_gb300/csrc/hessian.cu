// hessian.cu -- EAM Hessian, mass weighting and eigenvalues (compiled with -fmad=false).
//
// Restates EAM::hessian (src/potential/EAM/eam.cpp:122-233) on the device. Pass 1, one thread per atom
// b (active and frozen): rho_b = sum_a phi(t_a, t_b)(r) and mu_b = -sum_a phi'(t_a, t_b)(r) dr / r
// (A.13), with F'(rho_b) and F''(rho_b). Pass 2, one warp (CTA) per active atom z, writes only column block z
// of the dense 3n x 3n matrix (row-major; the rows of atom a are 3a..3a+2):
//   H(z,z) = F''_z mu_z mu_z^T + sum_a [A 1 - ABFpp dr dr^T]                           (A.15, A.14)
//   H(a,z) += -BArr dr dr^T - A 1 + ur dr mu_z^T - ru mu_a dr^T       for active a > z
//   H(g,z) -= F''_a phi'(t_z,t_a)(r) phi'(t_g,t_a)(r_ag) / (r r_ag) dr_ag dr^T
//             for every neighbour g of a that is active with g > z, or a periodic image of z itself.
// Neighbours come from the list in the reference's visiting order, every coefficient is formed in the
// reference's operation order, and every element receives its contributions in the reference's order:
// lane 0 adds the (z,z) and (a,z) terms of neighbour a, then the warp's lanes split a's neighbours g,
// so each (g,z) block takes the contributions of successive a in the order of the serial loop (equal g
// within one group of 32 are applied in list order, one occurrence per round). The result is the
// matrix the reference's loops build, bit for bit.
//
// Hessian::mass_weight (system/hessian.hpp:136-143) scales block (j, i) by 1/sqrt(m_i m_j), and
// Hessian::eigenvalues (system/hessian.hpp:86-93, Eigen's SelfAdjointEigenSolver on the lower
// triangle) becomes this library's dense symmetric eigensolver (eigen.cu) on the same triangle, applied
// to the active atoms' block only: frozen atoms' rows and columns are zero, so each frozen coordinate
// adds one exact zero eigenvalue.

#include <memory>

#include "internal.hpp"

namespace flygpu {

  namespace {

    struct Lookup {
      double x0;
      long long i;
    };

    // Spline::fetch (spline.hpp:135-154); out-of-range arguments report false.
    __device__ inline bool fetch(double x, double inv_dx, double dx, int n_spines, Lookup& o) {
      if (!(x >= 0)) return false;
      double const u = x * inv_dx;
      if (!(u < static_cast<double>(n_spines))) return false;
      o.i = static_cast<long long>(u);
      o.x0 = x - static_cast<double>(o.i) * dx;
      return true;
    }

    // Spline::f / fp / fpp (spline.hpp:100-123).
    __device__ inline double f_of(D4 const* __restrict__ tab, Lookup const& l) {
      D4 const c = tab[l.i];
      return c.x + l.x0 * (c.y + l.x0 * (c.z + l.x0 * c.w));
    }
    __device__ inline double fp_of(D4 const* __restrict__ tab, Lookup const& l) {
      D4 const c = tab[l.i];
      return c.y + l.x0 * (2.0 * c.z + l.x0 * 3.0 * c.w);
    }
    __device__ inline double fpp_of(D4 const* __restrict__ tab, Lookup const& l) {
      D4 const c = tab[l.i];
      return 2 * c.z + 6.0 * l.x0 * c.w;
    }

    // DataEAM::phi(a, b) / v(a, b): the function of neighbour type a at receiver type b.
    __device__ inline D4 const* phi_t(TablesView const& tb, std::uint32_t a, std::uint32_t b) {
      return tb.phi64 + static_cast<std::int64_t>(a + tb.n_types * b) * tb.nR;
    }
    __device__ inline D4 const* v_t(TablesView const& tb, std::uint32_t a, std::uint32_t b) {
      return tb.v64 + static_cast<std::int64_t>(a + tb.n_types * b) * tb.nR;
    }

    // Pass 1: rho, mu, F'(rho) and F''(rho) of every atom.
    __global__ void k_hess_rho(TablesView tb, std::int64_t n, long long const* __restrict__ offs,
                               int const* __restrict__ idx, double const* __restrict__ dr,
                               std::uint32_t const* __restrict__ types, double* __restrict__ rho_mu,
                               double* __restrict__ fder, int* __restrict__ err) {
      std::int64_t const b = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (b >= n) return;
      std::uint32_t const t_b = types[b];
      double rho = 0, m0 = 0, m1 = 0, m2 = 0;
      bool bad = false;
      for (long long k = offs[b]; k < offs[b + 1]; ++k) {
        double const x = dr[3 * k], y = dr[3 * k + 1], z = dr[3 * k + 2];
        double const r = sqrt((x * x + y * y) + z * z);
        Lookup l;
        if (!fetch(r, tb.inv_dR, tb.dR, tb.nR, l)) {
          bad = true;
          continue;
        }
        D4 const* ph = phi_t(tb, types[idx[k]], t_b);
        rho += f_of(ph, l);
        double const fp = fp_of(ph, l);
        m0 -= fp * x / r;
        m1 -= fp * y / r;
        m2 -= fp * z / r;
      }
      rho_mu[4 * b + 0] = rho;
      rho_mu[4 * b + 1] = m0;
      rho_mu[4 * b + 2] = m1;
      rho_mu[4 * b + 3] = m2;
      Lookup l;
      double fp = 0, fpp = 0;
      if (fetch(rho, tb.inv_dP, tb.dP, tb.nP, l)) {
        D4 const* Ft = tb.F64 + static_cast<std::int64_t>(t_b) * tb.nP;
        fp = fp_of(Ft, l);
        fpp = fpp_of(Ft, l);
      } else {
        bad = true;
      }
      fder[2 * b] = fp;
      fder[2 * b + 1] = fpp;
      if (bad) atomicOr(err, ERR_SPLINE_OOB);
    }

    // Pass 2: column block z, one 32-thread CTA per active atom (cols lists them), so the columns spread
    // over the SMs whatever the atoms' numbering.
    __global__ void __launch_bounds__(32)
        k_hess_col(TablesView tb, std::int64_t n, int const* __restrict__ cols, long long const* __restrict__ offs,
                   int const* __restrict__ idx, double const* __restrict__ dr, std::uint32_t const* __restrict__ types,
                   std::uint8_t const* __restrict__ frozen, double const* __restrict__ rho_mu,
                   double const* __restrict__ fder, double* __restrict__ H, int* __restrict__ err) {
      std::int64_t const z = cols[blockIdx.x];
      int const lane = threadIdx.x;
      if (z >= n || frozen[z]) return;
      std::int64_t const N = 3 * n;
      auto at = [&](std::int64_t i, std::int64_t j, int r, int c) -> double& { return H[(3 * i + r) * N + 3 * j + c]; };
      std::uint32_t const tz = types[z];
      double const mz[3] = {rho_mu[4 * z + 1], rho_mu[4 * z + 2], rho_mu[4 * z + 3]};
      double const fz_p = fder[2 * z], fz_pp = fder[2 * z + 1];
      bool bad = false;
      if (lane == 0)
        for (int r = 0; r < 3; ++r)
          for (int c = 0; c < 3; ++c) at(z, z, r, c) = (fz_pp * mz[r]) * mz[c];
      __syncwarp();
      for (long long k = offs[z]; k < offs[z + 1]; ++k) {
        std::int64_t const a = idx[k];
        double const d[3] = {dr[3 * k], dr[3 * k + 1], dr[3 * k + 2]};
        double const r = sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]);
        Lookup l;
        if (!fetch(r, tb.inv_dR, tb.dR, tb.nR, l)) {
          bad = true;
          continue;
        }
        std::uint32_t const ta = types[a];
        double const fa_p = fder[2 * a], fa_pp = fder[2 * a + 1];
        D4 const* p_az = phi_t(tb, ta, tz);
        D4 const* p_za = phi_t(tb, tz, ta);
        D4 const* v_az = v_t(tb, ta, tz);
        double const pza = fp_of(p_za, l);
        if (lane == 0) {
          double const A = (fp_of(v_az, l) + fz_p * fp_of(p_az, l) + fa_p * pza) / r;
          double const B = fpp_of(v_az, l) + fz_p * fpp_of(p_az, l) + fa_p * fpp_of(p_za, l);
          double const ABFpp = (A - B - fa_pp * (pza * pza)) / (r * r);
          for (int i = 0; i < 3; ++i)
            for (int c = 0; c < 3; ++c) at(z, z, i, c) += (i == c ? A : A * 0.0) - (ABFpp * d[i]) * d[c];
          if (a > z && !frozen[a]) {
            double const BArr = (B - A) / (r * r);
            double const ur = fz_pp * fp_of(p_az, l) / r;
            double const ru = fa_pp * pza / r;
            double const ma[3] = {rho_mu[4 * a + 1], rho_mu[4 * a + 2], rho_mu[4 * a + 3]};
            for (int i = 0; i < 3; ++i)
              for (int c = 0; c < 3; ++c)
                at(a, z, i, c) += (((-BArr * d[i]) * d[c] - (i == c ? A : A * 0.0)) + (ur * d[i]) * mz[c]) -
                                  (ru * ma[i]) * d[c];
          }
        }
        __syncwarp();
        double const ddFg = fa_pp * pza;
        long long const g0 = offs[a], g1 = offs[a + 1];
        for (long long base = g0; base < g1; base += 32) {
          long long const q = base + lane;
          bool const live = q < g1;
          std::int64_t g = -1;
          double e[3] = {0, 0, 0};
          double mag = 0;
          bool use = false;
          if (live) {
            g = idx[q];
            e[0] = dr[3 * q];
            e[1] = dr[3 * q + 1];
            e[2] = dr[3 * q + 2];
            double const sx = d[0] + e[0], sy = d[1] + e[1], sz = d[2] + e[2];
            use = (g > z && !frozen[g]) || (g == z && sqrt((sx * sx + sy * sy) + sz * sz) > 1e-6);
            if (use) {
              double const r_ag = sqrt((e[0] * e[0] + e[1] * e[1]) + e[2] * e[2]);
              Lookup m;
              if (fetch(r_ag, tb.inv_dR, tb.dR, tb.nR, m)) {
                mag = ddFg / (r * r_ag) * fp_of(phi_t(tb, types[g], ta), m);
              } else {
                bad = true;
                use = false;
              }
            }
          }
          // Equal g within the group (periodic images in small cells) are applied in list order.
          unsigned const peers = __match_any_sync(0xffffffffu, use ? g : -1 - lane);
          int const rank = __popc(peers & ((1u << lane) - 1u));
          int rounds = use ? rank + 1 : 0;
          for (int o = 16; o > 0; o >>= 1) rounds = max(rounds, __shfl_xor_sync(0xffffffffu, rounds, o));
          for (int round = 0; round < rounds; ++round) {
            if (use && rank == round)
              for (int i = 0; i < 3; ++i)
                for (int c = 0; c < 3; ++c) at(g, z, i, c) -= (mag * e[i]) * d[c];
            __syncwarp();
          }
        }
        __syncwarp();
      }
      if (__any_sync(0xffffffffu, bad) && lane == 0) atomicOr(err, ERR_SPLINE_OOB);
    }

    // Hessian::mass_weight: element (row, col) *= 1 / sqrt(m_col m_row), masses by atom.
    __global__ void k_mass_weight(double* __restrict__ H, std::int64_t N, double const* __restrict__ m3) {
      std::int64_t const e = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (e >= N * N) return;
      std::int64_t const row = e / N, col = e - row * N;
      H[e] *= 1 / sqrt(m3[col] * m3[row]);
    }

  }  // namespace

  // Dense 3n x 3n Hessian into d_H (device, row-major). Synchronises the list's stream.
  void eam_hessian(flygpu_eam const* E, flygpu_list* L, std::uint8_t const* h_frozen, double* d_H) {
    std::int64_t const n = L->n;
    cudaStream_t const s = L->stream;
    if (n == 0) return;
    HessianScratch& P = L->hs;
    std::vector<int> cols;
    for (std::int64_t i = 0; i < n; ++i)
      if (!h_frozen[i]) cols.push_back(static_cast<int>(i));
    // The column kernel skips frozen rows by the device flags: upload the same flags the active columns
    // come from, so rows and columns always agree.
    L->frozen.reserve(static_cast<std::size_t>(n) + 1);
    FLY_CUDA(cudaMemcpyAsync(L->frozen.p, h_frozen, static_cast<std::size_t>(n), cudaMemcpyHostToDevice, s));
    L->frozen_set = true;
    P.cols.reserve(std::max<std::size_t>(cols.size(), 1));
    if (!cols.empty())
      FLY_CUDA(cudaMemcpyAsync(P.cols.p, cols.data(), sizeof(int) * cols.size(), cudaMemcpyHostToDevice, s));
    P.offs.reserve(static_cast<std::size_t>(n) + 1);
    std::vector<int> const cnt = list_export_device(L, E->r_cut, P.offs, P.idx, P.dr);
    std::vector<long long> ho(static_cast<std::size_t>(n) + 1, 0);
    for (std::int64_t i = 0; i < n; ++i) ho[static_cast<std::size_t>(i) + 1] = ho[static_cast<std::size_t>(i)] + cnt[static_cast<std::size_t>(i)];
    FLY_CUDA(cudaMemcpyAsync(P.offs.p, ho.data(), sizeof(long long) * ho.size(), cudaMemcpyHostToDevice, s));
    P.rho_mu.reserve(4 * static_cast<std::size_t>(n));
    P.fder.reserve(2 * static_cast<std::size_t>(n));
    std::size_t const N = 3 * static_cast<std::size_t>(n);
    FLY_CUDA(cudaMemsetAsync(d_H, 0, sizeof(double) * N * N, s));
    TablesView const tb = E->view();
    // one warp per CTA: the per-atom binary64 work spreads over as many SMs as there are warps (binary64
    // throughput is per SM), each thread's arithmetic unchanged
    launch(k_hess_rho, static_cast<unsigned>((n + 31) / 32), 32, 0, s, tb, n, P.offs.p, P.idx.p, P.dr.p, L->types.p,
           P.rho_mu.p, P.fder.p, L->err.p);
    if (!cols.empty())
      launch(k_hess_col, static_cast<unsigned>(cols.size()), 32, 0, s, tb, n, P.cols.p, P.offs.p, P.idx.p, P.dr.p,
             L->types.p, L->frozen.p, P.rho_mu.p, P.fder.p, d_H, L->err.p);
    FLY_CUDA(cudaStreamSynchronize(s));  // the host vectors ho and cols stay alive until their copies have run
  }

  void hessian_mass_weight(flygpu_eam const* E, flygpu_list* L, double const* type_mass, std::uint32_t const* h_types,
                           double* d_H) {
    std::int64_t const n = L->n;
    if (n == 0) return;
    cudaStream_t const s = L->stream;
    std::vector<double> m3(3 * static_cast<std::size_t>(n));
    for (std::int64_t i = 0; i < n; ++i) {
      std::uint32_t const t = h_types[i];
      if (t >= static_cast<std::uint32_t>(E->n_types)) fail(FLYGPU_INVALID_ARG, "type index out of range");
      double const m = type_mass ? type_mass[t] : E->mass[t];
      if (!(m > 0)) fail(FLYGPU_INVALID_ARG, "masses must be positive");
      for (int k = 0; k < 3; ++k) m3[static_cast<std::size_t>(3 * i + k)] = m;
    }
    DevBuf<double>& dm = L->hs.m3;
    dm.reserve(m3.size());
    FLY_CUDA(cudaMemcpyAsync(dm.p, m3.data(), sizeof(double) * m3.size(), cudaMemcpyHostToDevice, s));
    std::int64_t const N = 3 * n;
    launch(k_mass_weight, static_cast<unsigned>((N * N + 255) / 256), 256, 0, s, d_H, N, dm.p);
    FLY_CUDA(cudaStreamSynchronize(s));
  }

  // Eigenvalues of a Hessian whose frozen atoms' rows and columns are zero: the matrix is block diagonal
  // (after a permutation) with the active coordinates' block and a zero block, so its spectrum is the
  // active block's eigenvalues and one exact zero per frozen coordinate. Only the active block is
  // diagonalised; the zeros are merged in ascending order. d_H (N x N, row-major lower triangle) is
  // left unchanged when some atoms are frozen.
  void hessian_eigenvalues(flygpu_list* L, double* d_H, std::uint8_t const* h_frozen, double* h_eig) {
    std::int64_t const n = L->n, N = 3 * n;
    std::vector<int> act;
    for (std::int64_t i = 0; i < n; ++i)
      if (!h_frozen[i])
        for (int k = 0; k < 3; ++k) act.push_back(static_cast<int>(3 * i + k));
    std::int64_t const M = static_cast<std::int64_t>(act.size());
    if (M == N) {
      dense_eigenvalues(L, d_H, N, {}, h_eig);
      return;
    }
    std::vector<double> w(static_cast<std::size_t>(M));
    if (M > 0) dense_eigenvalues(L, d_H, N, act, w.data());
    std::size_t const zeros = static_cast<std::size_t>(N - M);
    std::size_t j = 0, o = 0;
    while (j < w.size() && w[j] < 0) h_eig[o++] = w[j++];
    for (std::size_t z = 0; z < zeros; ++z) h_eig[o++] = 0.0;
    while (j < w.size()) h_eig[o++] = w[j++];
  }

}  // namespace flygpu
