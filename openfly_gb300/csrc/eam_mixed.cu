// eam_mixed.cu -- EAM energy and gradient with binary32 pair terms and binary64 accumulation.
//
// Same passes as EAM::energy / EAM::gradient (src/potential/EAM/eam.cpp:33-120). GB300 executes
// binary64 at about 1/64 of the binary32 rate, so every per-pair operation here is binary32. The
// operations whose single rounding would dominate the force error are carried as unevaluated binary32
// pairs (float-float), which costs binary32 instructions only:
//   * r^2 from the packed (hi, lo) offset coordinates: hi parts share one binade, so hi_n - hi_i is
//     exact (Sterbenz); the squares are split exactly with an FMA and summed with TwoSum, so r^2 is a
//     float-float good to ~2^-44 relative;
//   * the cut-off decision is the reference's binary64 `(dx*dx + dy*dy) + dz*dz < rc*rc` (list.hpp:139-154):
//     the float-float r^2 decides every pair outside a narrow band around rc^2 and the rare pairs inside
//     it take the binary64 test on the slots' binary64 positions;
//   * r = r0 + dl (one Newton correction of the binary32 square root), 1/r to binary32 accuracy, and the
//     table coordinate u = r / dR as a float-float, so the interval's unit coordinate t = u - i keeps
//     ~2^-40 absolute accuracy (a binary32 u near 5000 would keep only ~2^-12);
//   * the force pass's derivative records carry each slope coefficient as a binary32 pair and the pair
//     magnitude v' + F'_i phi'_{q->i} + F'_q phi'_{i->q} is combined with TwoProduct / TwoSum, because its
//     three terms partially cancel.
// Pair terms are summed in binary32 over runs of at most CHUNK consecutive neighbours and each run is
// added to the atom's binary64 accumulator (density, pair energy, gradient). F(rho) and F'(rho) are
// per-atom and evaluated in binary64 from the binary64 table. Against the binary64 reference this keeps
// the gradient within ~3e-7 norm-wise relative on a 431-atom vacancy cell with sigma = 0.02 A noise.
// Both passes are bound by L1/TEX gathers: each pair reads its neighbour's 32-byte slot record and one
// 32-byte spline record (value records in the density pass, derivative records in the force pass) with
// one 256-bit load each; the force pass reads a second record only for pairs of different types
// (phi of the other order).

#include <cmath>

#include "internal.hpp"
#include "ld256.cuh"

namespace flygpu {

  __global__ void k_energy_final(double const* __restrict__ part, int nparts, double* __restrict__ out);

  namespace {

    constexpr int T = 128;
    constexpr int CHUNK = 8;

    // The cut-off of one call: rc^2 in binary64 (the reference's test), as a binary32 pair, and the
    // half-width of the band around it inside which the float-float r^2 does not decide.
    struct Cut {
      double rc2;
      float rc2h, rc2l, band;
      float inv_h, inv_l;  // 1/dR as a binary32 pair
      int nR;
    };

    __device__ __forceinline__ float two_sum(float a, float b, float& e) {
      float const s = __fadd_rn(a, b);
      float const bb = __fsub_rn(s, a);
      e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
      return s;
    }

    struct PairGeo {
      float dx, dy, dz;  // r_q - r_i rounded to binary32
      float ir;          // 1 / r
      float t;           // unit coordinate in interval i
      int i;
    };

    // Geometry of the pair (i = me, q = the neighbour record oh/ol; p, q their physical slots). Returns
    // false when the pair is beyond the cut-off or its table coordinate is out of range (then sets bad).
    __device__ __forceinline__ bool pair_geometry(float4 const& oh, float4 const& ol, Packed const& me, Cut const& c,
                                                  D4 const* __restrict__ pos, int p, int q, PairGeo& g, bool& bad) {
      float const xh = __fsub_rn(oh.x, me.hx), yh = __fsub_rn(oh.y, me.hy), zh = __fsub_rn(oh.z, me.hz);
      float const xl = __fsub_rn(ol.x, me.lx), yl = __fsub_rn(ol.y, me.ly), zl = __fsub_rn(ol.z, me.lz);
      // r^2 = sum (h + l)^2 as s2 + r2l
      float const px = __fmul_rn(xh, xh), py = __fmul_rn(yh, yh), pz = __fmul_rn(zh, zh);
      float const ex = fmaf(xh, xh, -px), ey = fmaf(yh, yh, -py), ez = fmaf(zh, zh, -pz);
      float e1, e2;
      float const s1 = two_sum(px, py, e1);
      float const s2 = two_sum(s1, pz, e2);
      float const cr = fmaf(xh, xl, fmaf(yh, yl, __fmul_rn(zh, zl)));
      float const r2l = __fadd_rn(__fadd_rn(__fadd_rn(ex, ey), __fadd_rn(ez, e1)), fmaf(2.f, cr, e2));
      float const D = __fadd_rn(__fsub_rn(s2, c.rc2h), __fsub_rn(r2l, c.rc2l));
      if (D >= c.band) return false;
      if (D > -c.band) {
        D4 const a = pos[p], b = pos[q];
        double const dx = __dsub_rn(b.x, a.x), dy = __dsub_rn(b.y, a.y), dz = __dsub_rn(b.z, a.z);
        if (!(__dadd_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)), __dmul_rn(dz, dz)) < c.rc2)) return false;
      }
      // r = r0 + dl and 1/r
      float const ir0 = rsqrtf(s2);
      float const r0 = __fmul_rn(s2, ir0);
      float const res = __fadd_rn(fmaf(-r0, r0, s2), r2l);
      float const dl = __fmul_rn(res, __fmul_rn(0.5f, ir0));
      g.ir = fmaf(ir0, fmaf(-dl, ir0, fmaf(-r0, ir0, 1.f)), ir0);
      // u = r / dR as uh + ul
      float const uh = __fmul_rn(r0, c.inv_h);
      float const ul = fmaf(r0, c.inv_l, fmaf(dl, c.inv_h, fmaf(r0, c.inv_h, -uh)));
      if (!(uh >= 0.f) || !(uh < static_cast<float>(c.nR))) {
        bad = true;
        return false;
      }
      g.i = static_cast<int>(uh);
      g.t = __fadd_rn(__fsub_rn(uh, static_cast<float>(g.i)), ul);
      g.dx = __fadd_rn(xh, xl);
      g.dy = __fadd_rn(yh, yl);
      g.dz = __fadd_rn(zh, zl);
      return true;
    }

    __device__ inline float f32(float4 c, float t) { return c.x + t * (c.y + t * (c.z + t * c.w)); }
    // b_lo + t (2c + 3 t d) of a derivative record (its b_hi is added by the caller)
    __device__ inline float dtail32(float4 c, float t) { return fmaf(t, fmaf(t, c.w, c.z), c.y); }

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
                                                     D4 const* __restrict__ pos, int const* __restrict__ pimg,
                                                     int const* __restrict__ real_phys, int const* __restrict__ nbr,
                                                     int const* __restrict__ ncount, std::int64_t n, Cut c,
                                                     double* __restrict__ fprime, double* __restrict__ part,
                                                     int* __restrict__ err) {
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
            PairGeo g;
            if (pair_geometry(oh, ol, me, c, pos, p, q, g, bad)) {
              int const tq = __float_as_int(oh.w);
              float4 cphi, cv;
              ld256(tb.pv32 + static_cast<std::int64_t>(ti * nt + tq) * tb.nR + g.i, cphi, cv);
              rho_f += f32(cphi, g.t);
              if (ENERGY) v_f += f32(cv, g.t);
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
          D4 const cf = tb.F64[static_cast<std::int64_t>(ti) * tb.nP + i];
          fpv = cf.y + x0 * (2.0 * cf.z + x0 * 3.0 * cf.w);
          if (ENERGY) femb = cf.x + x0 * (cf.y + x0 * (cf.z + x0 * cf.w));
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
                                                   D4 const* __restrict__ pos, int const* __restrict__ pimg,
                                                   int const* __restrict__ real_phys, int const* __restrict__ nbr,
                                                   int const* __restrict__ ncount, std::int64_t n, Cut c,
                                                   std::uint8_t const* __restrict__ frozen, double* __restrict__ grad,
                                                   int* __restrict__ err) {
      std::int64_t const j = static_cast<std::int64_t>(blockIdx.x) * T + threadIdx.x;
      if (j >= n) return;
      int const p = real_phys[j];
      std::int64_t const gi = pimg[p];
      double gx = 0, gy = 0, gz = 0;
      if (!frozen[gi]) {
        Packed const me = pk[p];
        int const ti = static_cast<int>(me.type);
        int const nt = tb.n_types;
        float const fi = me.fp;
        bool bad = false;
        int const cnt = ncount[j];
        for (int k0 = 0; k0 < cnt; k0 += CHUNK) {
          int const k1 = min(cnt, k0 + CHUNK);
          float fx = 0.f, fy = 0.f, fz = 0.f;
          for (int k = k0; k < k1; ++k) {
            int const q = nbr[static_cast<std::int64_t>(k) * n + j];
            float4 oh, ol;  // (hx, hy, hz, type bits), (lx, ly, lz, fp)
            ld256(pk + q, oh, ol);
            PairGeo g;
            if (pair_geometry(oh, ol, me, c, pos, p, q, g, bad)) {
              int const tq = __float_as_int(oh.w);
              // v' and phi'_{q->i} from the (t_i, t_q) record; phi'_{i->q} is the same function when the
              // types agree, else the phi' of the (t_q, t_i) record (v is symmetric in the types)
              float4 av, aq;
              ld256(tb.dv32 + static_cast<std::int64_t>(ti * nt + tq) * tb.nR + g.i, av, aq);
              float4 ao = aq;
              if (tq != ti) {
                float4 unused;
                ld256(tb.dv32 + static_cast<std::int64_t>(tq * nt + ti) * tb.nR + g.i, unused, ao);
              }
              float const fq = ol.w;
              // v' + F'_i phi'_{q->i} + F'_q phi'_{i->q} (per unit t): leading terms exactly, tails after
              float e1, e2, s1e, s2e;
              float const p1 = __fmul_rn(fi, aq.x), p2 = __fmul_rn(fq, ao.x);
              e1 = fmaf(fi, aq.x, -p1);
              e2 = fmaf(fq, ao.x, -p2);
              float const s1 = two_sum(av.x, p1, s1e);
              float const s2 = two_sum(s1, p2, s2e);
              float const tail = __fadd_rn(__fadd_rn(__fadd_rn(dtail32(av, g.t), fmaf(fi, dtail32(aq, g.t), e1)),
                                                     fmaf(fq, dtail32(ao, g.t), e2)),
                                           __fadd_rn(s1e, s2e));
              float const mag = __fadd_rn(s2, tail);
              float const s = __fmul_rn(__fmul_rn(mag, c.inv_h), g.ir);
              fx = fmaf(-s, g.dx, fx);
              fy = fmaf(-s, g.dy, fy);
              fz = fmaf(-s, g.dz, fz);
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

    // The cut-off of a call with the list's binary32 offset coordinates: the band covers the error of
    // the float-float r^2 (lo parts rounded at 2^-24 of the hi binade's ulp, float-float sums at ~2^-44)
    // with a margin of 8.
    Cut make_cut(flygpu_eam const* E, flygpu_list const* L) {
      Cut c{};
      double const rc = E->r_cut;
      c.rc2 = rc * rc;
      c.rc2h = static_cast<float>(c.rc2);
      c.rc2l = static_cast<float>(c.rc2 - static_cast<double>(c.rc2h));
      double ulp_hi = 0;
      for (int k = 0; k < 3; ++k) ulp_hi = std::max(ulp_hi, std::ldexp(1.0, std::ilogb(L->shift[k] + L->g.L[k]) - 23));
      double const e_dx = 4.0 * std::ldexp(ulp_hi, -24);
      double const e_r2 = 2.0 * std::sqrt(3.0) * L->g.rc * e_dx + std::ldexp(c.rc2, -40);
      c.band = static_cast<float>(8.0 * e_r2 + std::ldexp(c.rc2, -44));
      TablesView const tb = E->view();
      c.inv_h = tb.finv_dR;
      c.inv_l = tb.finv_dR_lo;
      c.nR = tb.nR;
      return c;
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
    Cut const c = make_cut(E, L);
    unsigned const nb = static_cast<unsigned>((n + T - 1) / T);
    L->fprime.reserve(static_cast<std::size_t>(n));
    cudaEvent_t const t0 = timer_record(L);
    if (d_energy) {
      L->energy_part.reserve(2 * static_cast<std::size_t>(nb));
      launch(k_density32<true>, nb, T, 0, s, tb, L->packed.p, L->pos.p, L->pimg.p, L->real_phys.p, L->nbr.p, L->ncount.p,
                                         n, c, L->fprime.p, L->energy_part.p, L->err.p);
      launch(k_energy_final, 1, 256, 0, s, L->energy_part.p, static_cast<int>(nb), d_energy);
    } else {
      launch(k_density32<false>, nb, T, 0, s, tb, L->packed.p, L->pos.p, L->pimg.p, L->real_phys.p, L->nbr.p, L->ncount.p,
                                          n, c, L->fprime.p, nullptr, L->err.p);
    }
    timer_mark(L, TK_DENSITY, t0, timer_record(L));
    if (!d_grad) return;
    launch(k_fprime_packed, static_cast<unsigned>((L->n_slots + 255) / 256), 256, 0, s, L->packed.p, L->pimg.p, L->n_slots,
                                                                                    L->fprime.p);
    cudaEvent_t const t1 = timer_record(L);
    launch(k_force32, nb, T, 0, s, tb, L->packed.p, L->pos.p, L->pimg.p, L->real_phys.p, L->nbr.p, L->ncount.p, n, c,
                               L->frozen.p, d_grad, L->err.p);
    timer_mark(L, TK_FORCE, t1, timer_record(L));
  }

}  // namespace flygpu
