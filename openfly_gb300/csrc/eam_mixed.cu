// eam_mixed.cu -- EAM energy and gradient with binary32 pair terms and binary64 accumulation.
//
// Same passes as EAM::energy / EAM::gradient (src/potential/EAM/eam.cpp:33-120). GB300 executes
// binary64 at about 1/70 of the binary32 rate, so every per-pair operation here is binary32:
//   * dr from the packed (hi, lo) offset coordinates: hi parts share one binade, so hi_n - hi_i is
//     exact (Sterbenz) and dr carries one binary32 rounding, like a binary64 dr rounded to binary32;
//   * spline lookups use binary32 coefficients in the interval's unit coordinate t = r/dr - i;
//   * pair terms are summed in binary32 over runs of at most CHUNK consecutive neighbours and each run
//     is added to the atom's binary64 accumulator (density, pair energy, gradient).
// F(rho) and F'(rho) are per-atom and evaluated in binary64 from the binary64 table.
// Both passes are bound by L1/TEX gathers, so each pair reads its neighbour's 32-byte slot record and
// one merged 32-byte spline record (phi and v of the ordered type pair) with one 256-bit load each; the
// force pass reads a second merged record only for pairs of different types (phi of the other order).

#include "internal.hpp"
#include "ld256.cuh"

namespace flygpu {

  __global__ void k_energy_final(double const* __restrict__ part, int nparts, double* __restrict__ out);

  namespace {

    constexpr int T = 128;
    constexpr int CHUNK = 8;

    __device__ inline bool fetch32(float r, float inv_dx, int n_spines, int& i, float& t) {
      float const u = r * inv_dx;
      if (!(u >= 0.f) || !(u < static_cast<float>(n_spines))) return false;
      i = static_cast<int>(u);
      t = u - static_cast<float>(i);
      return true;
    }

    __device__ inline float f32(float4 c, float t) { return c.x + t * (c.y + t * (c.z + t * c.w)); }
    __device__ inline float dfdt32(float4 c, float t) { return c.y + t * (2.f * c.z + 3.f * t * c.w); }

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
    __global__ void __launch_bounds__(T) k_density32(TablesView tb, Packed const* __restrict__ pk,
                                                     int const* __restrict__ pimg, int const* __restrict__ real_phys,
                                                     int const* __restrict__ nbr, int const* __restrict__ ncount,
                                                     std::int64_t n, float rc2, double* __restrict__ fprime,
                                                     double* __restrict__ part, int* __restrict__ err) {
      std::int64_t const j = static_cast<std::int64_t>(blockIdx.x) * T + threadIdx.x;
      double vsum = 0, femb = 0;
      if (j < n) {
        int const p = real_phys[j];
        Packed const me = pk[p];
        int const ti = static_cast<int>(me.type);
        int const nt = tb.n_types;
        double rho = 0;
        float rho_f = 0.f, v_f = 0.f;
        bool bad = false;
        int const cnt = ncount[j];
        for (int k0 = 0; k0 < cnt; k0 += CHUNK) {
          int const k1 = min(cnt, k0 + CHUNK);
          for (int k = k0; k < k1; ++k) {
            int const q = nbr[static_cast<std::int64_t>(k) * n + j];
            float4 oh, ol;  // (hx, hy, hz, type bits), (lx, ly, lz, fp)
            ld256(pk + q, oh, ol);
            float const dx = (oh.x - me.hx) + (ol.x - me.lx);
            float const dy = (oh.y - me.hy) + (ol.y - me.ly);
            float const dz = (oh.z - me.hz) + (ol.z - me.lz);
            float const r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < rc2) {
              float const r = sqrtf(r2);
              int const tq = __float_as_int(oh.w);
              int i;
              float t;
              if (!fetch32(r, tb.finv_dR, tb.nR, i, t)) {
                bad = true;
                continue;
              }
              float4 cphi, cv;
              ld256(tb.pv32 + static_cast<std::int64_t>(ti * nt + tq) * tb.nR + i, cphi, cv);
              rho_f += f32(cphi, t);
              if (ENERGY) v_f += f32(cv, t);
            }
          }
          rho += static_cast<double>(rho_f);
          rho_f = 0.f;
          if (ENERGY) {
            vsum += static_cast<double>(v_f);
            v_f = 0.f;
          }
        }
        double fpv = 0;
        double const u = rho * tb.inv_dP;
        if (rho >= 0 && u < static_cast<double>(tb.nP)) {
          long long const i = static_cast<long long>(u);
          double const x0 = rho - static_cast<double>(i) * tb.dP;
          D4 const c = tb.F64[static_cast<std::int64_t>(ti) * tb.nP + i];
          fpv = c.y + x0 * (2.0 * c.z + x0 * 3.0 * c.w);
          if (ENERGY) femb = c.x + x0 * (c.y + x0 * (c.z + x0 * c.w));
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

    __global__ void k_fprime_packed(Packed* __restrict__ pk, int const* __restrict__ pimg, std::int64_t slots,
                                    double const* __restrict__ fprime) {
      std::int64_t const p = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
      if (p < slots) pk[p].fp = static_cast<float>(fprime[pimg[p]]);
    }

    __global__ void __launch_bounds__(T) k_force32(TablesView tb, Packed const* __restrict__ pk,
                                                   int const* __restrict__ pimg, int const* __restrict__ real_phys,
                                                   int const* __restrict__ nbr, int const* __restrict__ ncount,
                                                   std::int64_t n, float rc2, std::uint8_t const* __restrict__ frozen,
                                                   double* __restrict__ grad, int* __restrict__ err) {
      std::int64_t const j = static_cast<std::int64_t>(blockIdx.x) * T + threadIdx.x;
      if (j >= n) return;
      int const p = real_phys[j];
      std::int64_t const gi = pimg[p];
      double gx = 0, gy = 0, gz = 0;
      if (!frozen[gi]) {
        Packed const me = pk[p];
        int const ti = static_cast<int>(me.type);
        int const nt = tb.n_types;
        float const inv = tb.finv_dR;
        bool bad = false;
        int const cnt = ncount[j];
        for (int k0 = 0; k0 < cnt; k0 += CHUNK) {
          int const k1 = min(cnt, k0 + CHUNK);
          float fx = 0.f, fy = 0.f, fz = 0.f;
          for (int k = k0; k < k1; ++k) {
            int const q = nbr[static_cast<std::int64_t>(k) * n + j];
            float4 oh, ol;  // (hx, hy, hz, type bits), (lx, ly, lz, fp)
            ld256(pk + q, oh, ol);
            float const dx = (oh.x - me.hx) + (ol.x - me.lx);
            float const dy = (oh.y - me.hy) + (ol.y - me.ly);
            float const dz = (oh.z - me.hz) + (ol.z - me.lz);
            float const r2 = dx * dx + dy * dy + dz * dz;
            if (r2 < rc2) {
              float const ir = rsqrtf(r2);
              float const r = r2 * ir;
              int const tq = __float_as_int(oh.w);
              int i;
              float t;
              if (!fetch32(r, inv, tb.nR, i, t)) {
                bad = true;
                continue;
              }
              // phi_{q->i} and v from the (t_i, t_q) record; phi_{i->q} is the same function when the
              // types agree, else the phi of the (t_q, t_i) record (v is symmetric in the types)
              float4 cphi, cv;
              ld256(tb.pv32 + static_cast<std::int64_t>(ti * nt + tq) * tb.nR + i, cphi, cv);
              float4 cphi_o = cphi;
              if (tq != ti) {
                float4 unused;
                ld256(tb.pv32 + static_cast<std::int64_t>(tq * nt + ti) * tb.nR + i, cphi_o, unused);
              }
              float const dv = dfdt32(cv, t);
              float const dphi_qi = dfdt32(cphi, t);
              float const dphi_iq = dfdt32(cphi_o, t);
              float const s = (dv + me.fp * dphi_qi + ol.w * dphi_iq) * inv * ir;
              fx -= s * dx;
              fy -= s * dy;
              fz -= s * dz;
            }
          }
          gx += static_cast<double>(fx);
          gy += static_cast<double>(fy);
          gz += static_cast<double>(fz);
        }
        if (bad) atomicOr(err, ERR_SPLINE_OOB);
      }
      grad[3 * gi + 0] = gx;
      grad[3 * gi + 1] = gy;
      grad[3 * gi + 2] = gz;
    }

  }  // namespace

  void eam_mixed(flygpu_eam const* E, flygpu_list* L, double* d_energy, double* d_grad) {
    std::int64_t const n = L->n;
    cudaStream_t const s = L->stream;
    double const rc = E->r_cut;
    if (rc > L->g.rc) fail(FLYGPU_INVALID_ARG, "potential r_cut is bigger than the list's cut-off");
    if (n == 0) {
      if (d_energy) FLY_CUDA(cudaMemsetAsync(d_energy, 0, sizeof(double), s));
      return;
    }
    list_pack(L);
    TablesView const tb = E->view();
    float const rc2 = static_cast<float>(rc * rc);
    unsigned const nb = static_cast<unsigned>((n + T - 1) / T);
    L->fprime.reserve(static_cast<std::size_t>(n));
    cudaEvent_t const t0 = timer_record(L);
    if (d_energy) {
      L->energy_part.reserve(2 * static_cast<std::size_t>(nb));
      launch(k_density32<true>, nb, T, 0, s, tb, L->packed.p, L->pimg.p, L->real_phys.p, L->nbr.p, L->ncount.p, n, rc2,
                                         L->fprime.p, L->energy_part.p, L->err.p);
      launch(k_energy_final, 1, 256, 0, s, L->energy_part.p, static_cast<int>(nb), d_energy);
    } else {
      launch(k_density32<false>, nb, T, 0, s, tb, L->packed.p, L->pimg.p, L->real_phys.p, L->nbr.p, L->ncount.p, n, rc2,
                                          L->fprime.p, nullptr, L->err.p);
    }
    timer_mark(L, TK_DENSITY, t0, timer_record(L));
    if (!d_grad) return;
    launch(k_fprime_packed, static_cast<unsigned>((L->n_slots + 255) / 256), 256, 0, s, L->packed.p, L->pimg.p, L->n_slots,
                                                                                    L->fprime.p);
    cudaEvent_t const t1 = timer_record(L);
    launch(k_force32, nb, T, 0, s, tb, L->packed.p, L->pimg.p, L->real_phys.p, L->nbr.p, L->ncount.p, n, rc2, L->frozen.p,
                               d_grad, L->err.p);
    timer_mark(L, TK_FORCE, t1, timer_record(L));
  }

}  // namespace flygpu
