// eam_fp64.cu -- EAM energy and gradient in binary64 (compiled with -fmad=false).
//
// Restates EAM::energy / EAM::gradient (src/potential/EAM/eam.cpp:33-120): a density pass
//   rho_b = sum_a phi(type_a, type_b)(r_ab),  F'_b = F_b'(rho_b)     (eam.cpp:62-86)
// then a force pass over active atoms
//   grad_g = -sum_a [v'(r) + F'_g phi'(t_a,t_g)(r) + F'_a phi'(t_g,t_a)(r)] / r * dr   (eam.cpp:90-119)
// with spline lookups as Spline::fetch/f/fp (utility/spline.hpp:81-154). One thread per real atom in
// cell order walks its neighbour column in the reference's visiting order, so rho, F' and the
// gradient are the same binary64 values the reference's loops produce. The energy is reduced per
// block and then by one block in a fixed order (run-to-run deterministic).

#include "internal.hpp"

namespace flygpu {

  namespace {

    constexpr int T = 128;

    struct Lookup {
      double x0;
      long long i;
    };

    // Spline::fetch (spline.hpp:135-154). Out-of-range arguments set ERR_SPLINE_OOB and evaluate 0.
    __device__ inline bool fetch(double x, double inv_dx, double dx, int n_spines, Lookup& o) {
      if (!(x >= 0)) return false;
      double const u = x * inv_dx;
      if (!(u < static_cast<double>(n_spines))) return false;
      o.i = static_cast<long long>(u);
      o.x0 = x - static_cast<double>(o.i) * dx;
      return true;
    }

    __device__ inline double f_of(D4 const* __restrict__ tab, Lookup const& l) {
      D4 const c = tab[l.i];
      return c.x + l.x0 * (c.y + l.x0 * (c.z + l.x0 * c.w));
    }

    __device__ inline double fp_of(D4 const* __restrict__ tab, Lookup const& l) {
      D4 const c = tab[l.i];
      return c.y + l.x0 * (2.0 * c.z + l.x0 * 3.0 * c.w);
    }

    __device__ double block_sum(double v) {
      __shared__ double sh[T / 32];
      for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
      int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      if (lane == 0) sh[warp] = v;
      __syncthreads();
      double s = 0;
      if (threadIdx.x == 0)
        for (int w = 0; w < T / 32; ++w) s += sh[w];
      __syncthreads();
      return s;
    }

    template <bool ENERGY>
    __global__ void __launch_bounds__(T) k_density(TablesView tb, D4 const* __restrict__ pos,
                                                   int const* __restrict__ ptype, int const* __restrict__ pimg,
                                                   int const* __restrict__ real_phys, int const* __restrict__ nbr,
                                                   int const* __restrict__ ncount, std::int64_t n, double rc2,
                                                   double* __restrict__ fprime, double* __restrict__ part,
                                                   int* __restrict__ err) {
      std::int64_t const j = static_cast<std::int64_t>(blockIdx.x) * T + threadIdx.x;
      double vsum = 0, femb = 0;
      if (j < n) {
        int const p = real_phys[j];
        D4 const ri = pos[p];
        int const ti = ptype[p];
        int const nt = tb.n_types;
        double rho = 0;
        bool bad = false;
        int const cnt = ncount[j];
        for (int k = 0; k < cnt; ++k) {
          int const q = nbr[static_cast<std::int64_t>(k) * n + j];
          D4 const rq = pos[q];
          double const dx = rq.x - ri.x, dy = rq.y - ri.y, dz = rq.z - ri.z;
          double const r2 = (dx * dx + dy * dy) + dz * dz;
          if (r2 < rc2) {
            double const r = sqrt(r2);
            int const tq = ptype[q];
            Lookup l;
            if (!fetch(r, tb.inv_dR, tb.dR, tb.nR, l)) {
              bad = true;
              continue;
            }
            if (ENERGY) vsum += f_of(tb.v64 + static_cast<std::int64_t>(ti + nt * tq) * tb.nR, l);
            rho += f_of(tb.phi64 + static_cast<std::int64_t>(tq + nt * ti) * tb.nR, l);
          }
        }
        Lookup l;
        double fpv = 0;
        if (fetch(rho, tb.inv_dP, tb.dP, tb.nP, l)) {
          D4 const* Ft = tb.F64 + static_cast<std::int64_t>(ti) * tb.nP;
          fpv = fp_of(Ft, l);
          if (ENERGY) femb = f_of(Ft, l);
        } else {
          bad = true;
        }
        fprime[pimg[p]] = fpv;
        if (bad) atomicOr(err, ERR_SPLINE_OOB);
      }
      if (ENERGY) {
        double const a = block_sum(vsum);
        double const b = block_sum(femb);
        if (threadIdx.x == 0) {
          part[2 * blockIdx.x + 0] = a;
          part[2 * blockIdx.x + 1] = b;
        }
      }
    }

    __global__ void k_fprime_slots(D4* __restrict__ pos, int const* __restrict__ pimg, std::int64_t slots,
                                   double const* __restrict__ fprime) {
      std::int64_t const p = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (p < slots) pos[p].w = fprime[pimg[p]];
    }

    __global__ void __launch_bounds__(T) k_force(TablesView tb, D4 const* __restrict__ pos,
                                                 int const* __restrict__ ptype, int const* __restrict__ pimg,
                                                 int const* __restrict__ real_phys, int const* __restrict__ nbr,
                                                 int const* __restrict__ ncount, std::int64_t n, double rc2,
                                                 std::uint8_t const* __restrict__ frozen, double* __restrict__ grad,
                                                 int* __restrict__ err) {
      std::int64_t const j = static_cast<std::int64_t>(blockIdx.x) * T + threadIdx.x;
      if (j >= n) return;
      int const p = real_phys[j];
      std::int64_t const i = pimg[p];
      double gx = 0, gy = 0, gz = 0;
      if (!frozen[i]) {
        D4 const ri = pos[p];
        int const ti = ptype[p];
        int const nt = tb.n_types;
        double const fpi = ri.w;
        bool bad = false;
        int const cnt = ncount[j];
        for (int k = 0; k < cnt; ++k) {
          int const q = nbr[static_cast<std::int64_t>(k) * n + j];
          D4 const rq = pos[q];
          double const dx = rq.x - ri.x, dy = rq.y - ri.y, dz = rq.z - ri.z;
          double const r2 = (dx * dx + dy * dy) + dz * dz;
          if (r2 < rc2) {
            double const r = sqrt(r2);
            int const tq = ptype[q];
            Lookup l;
            if (!fetch(r, tb.inv_dR, tb.dR, tb.nR, l)) {
              bad = true;
              continue;
            }
            double const mag = fp_of(tb.v64 + static_cast<std::int64_t>(tq + nt * ti) * tb.nR, l) +
                               fpi * fp_of(tb.phi64 + static_cast<std::int64_t>(tq + nt * ti) * tb.nR, l) +
                               rq.w * fp_of(tb.phi64 + static_cast<std::int64_t>(ti + nt * tq) * tb.nR, l);
            double const s = mag / r;
            gx -= s * dx;
            gy -= s * dy;
            gz -= s * dz;
          }
        }
        if (bad) atomicOr(err, ERR_SPLINE_OOB);
      }
      grad[3 * i + 0] = gx;
      grad[3 * i + 1] = gy;
      grad[3 * i + 2] = gz;
    }

  }  // namespace

  // Final energy: 0.5 * sum v + sum F over block partials, one block, fixed order.
  __global__ void k_energy_final(double const* __restrict__ part, int nparts, double* __restrict__ out) {
    __shared__ double sv[256], sf[256];
    double v = 0, f = 0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x) {
      v += part[2 * b];
      f += part[2 * b + 1];
    }
    sv[threadIdx.x] = v;
    sf[threadIdx.x] = f;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
      if (threadIdx.x < s) {
        sv[threadIdx.x] += sv[threadIdx.x + s];
        sf[threadIdx.x] += sf[threadIdx.x + s];
      }
      __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = (0.5 * sv[0]) + sf[0];
  }

  void eam_fp64(flygpu_eam const* E, flygpu_list* L, double* d_energy, double* d_grad) {
    std::int64_t const n = L->n;
    cudaStream_t const s = L->stream;
    double const rc = E->r_cut;
    if (rc > L->g.rc) fail(FLYGPU_INVALID_ARG, "potential r_cut is bigger than the list's cut-off");
    if (n == 0) {
      if (d_energy) FLY_CUDA(cudaMemsetAsync(d_energy, 0, sizeof(double), s));
      return;
    }
    TablesView const tb = E->view();
    double const rc2 = rc * rc;
    unsigned const nb = static_cast<unsigned>((n + T - 1) / T);
    L->fprime.reserve(static_cast<std::size_t>(n));
    cudaEvent_t const t0 = timer_record(L);
    if (d_energy) {
      L->energy_part.reserve(2 * static_cast<std::size_t>(nb));
      launch(k_density<true>, nb, T, 0, s, tb, L->pos.p, L->ptype.p, L->pimg.p, L->real_phys.p, L->nbr.p, L->ncount.p, n, rc2,
                                       L->fprime.p, L->energy_part.p, L->err.p);
      launch(k_energy_final, 1, 256, 0, s, L->energy_part.p, static_cast<int>(nb), d_energy);
    } else {
      launch(k_density<false>, nb, T, 0, s, tb, L->pos.p, L->ptype.p, L->pimg.p, L->real_phys.p, L->nbr.p, L->ncount.p, n,
                                        rc2, L->fprime.p, nullptr, L->err.p);
    }
    timer_mark(L, TK_DENSITY, t0, timer_record(L));
    if (!d_grad) return;
    launch(k_fprime_slots, static_cast<unsigned>((L->n_slots + 255) / 256), 256, 0, s, L->pos.p, L->pimg.p, L->n_slots,
                                                                                   L->fprime.p);
    cudaEvent_t const t1 = timer_record(L);
    launch(k_force, nb, T, 0, s, tb, L->pos.p, L->ptype.p, L->pimg.p, L->real_phys.p, L->nbr.p, L->ncount.p, n, rc2,
                             L->frozen.p, d_grad, L->err.p);
    timer_mark(L, TK_FORCE, t1, timer_record(L));
  }

}  // namespace flygpu
