// search_kernel.cuh -- batched, resumable dimer searches and L-BFGS minimisations, one CTA per search.
//
// Device restatement of the reference's search stack for many independent searches at once:
//   Dimer::find_sp         src/saddle/dimer.cpp:28-171
//   Rotor::eff_gradient    src/saddle/rotor.cpp:49-164 (trans_proj rotor.cpp:33-47)
//   StepLBFGS::newton_step src/minimise/LBFGS/lbfgs_core.cpp:29-87
//   LBFGS::minimise        src/minimise/LBFGS/lbfgs.cpp:29-115
//   EAM::gradient/energy   src/potential/EAM/eam.cpp:33-120 over a per-search neighbour list
// A persistent grid pulls searches from an atomic work counter (largest first). Inside the CTA that
// owns a search, the neighbour build and the EAM passes use every thread; the search's vector
// algebra and control (two-loop recursions, dots, rotor angles, trust radius) run in warp 0 alone,
// with warp-level binary64 reductions and no block barriers, and warp 0 passes its decisions to the
// other warps through shared memory. GB300 issues binary64 at ~1/70 of binary32, so keeping the
// scalar and vector binary64 work to one warp (and transcendental scalars to one lane) is what keeps
// the search off the binary64 pipe.
// Vectors are compacted to mobile atoms (not frozen, or with a non-zero axis component): the
// reference's vectors are exactly zero elsewhere, so the compacted algebra is the same algebra.
// State lives in global memory (L2-resident while the search runs) and is saved at translation-step
// boundaries, so a launch can stop after `budget` steps and a later launch resumes the search.
// Kernels never trap and never wait on other CTAs: errors set the search's status and end it.

#pragma once

#include <type_traits>

#include "search.hpp"

namespace flygpu {

  namespace {

    constexpr unsigned FULL = 0xffffffffu;
    constexpr int U = 4;    // neighbours per group in the gradient's binary32 pair walks (rho_walk32)
    constexpr int U64 = 2;  // the same for the binary64 walks (twice the registers per neighbour)
    // Packed::type of a search's records: the atom type, with MOBILE_BIT set for mobile atoms.
    constexpr std::uint32_t TYPE_MASK = 0xffu, MOBILE_BIT = 0x100u;
    // Fixed-point scale of the static atoms' density accumulators (Ctx::dacc): 2^32 for binary32 terms,
    // 2^40 for binary64 terms. Integer sums are exact and independent of the order of the atomics.
    template <bool MIXED>
    __device__ constexpr double dacc_scale() {
      return MIXED ? 4294967296.0 : 1099511627776.0;
    }

    enum : int { F_OOB = 1, F_NLIST = 2 };
    enum : int { ACT_GO = 0, ACT_REBUILD = 1, ACT_STOP = 2 };

    struct Blk {
      double red[32];
      double rhoR[MAX_HIST], alphaR[MAX_HIST];
      double rhoT[MAX_HIST], alphaT[MAX_HIST];  // the translation L-BFGS scalars, staged from SearchDev
      double curv;
      int n_need;  // atoms in the current needed list
      int item;
      int flag;    // error bits (F_OOB, F_NLIST), any thread
      int action;  // warp 0 -> block
    };

    __device__ inline double warp_sum(double v) {
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
      return v;
    }

    // Block-wide sum (all threads receive it); only used for the final energy.
    __device__ inline double block_sum(double v, Blk& sh) {
      int const lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
      v = warp_sum(v);
      __syncthreads();
      if (lane == 0) sh.red[w] = v;
      __syncthreads();
      double s = 0;
      for (int k = 0; k < nw; ++k) s += sh.red[k];
      __syncthreads();
      return s;
    }

    // Scalar evaluated on lane 0 of the calling warp and broadcast (binary64 transcendentals and
    // divisions cost dozens of binary64 instructions each).
    template <typename F>
    __device__ inline double lane0(F&& f) {
      double v = 0;
      if ((threadIdx.x & 31) == 0) v = f();
      return __shfl_sync(FULL, v, 0);
    }

    struct Ctx {
      SearchDev* S;
      int n, na, M, mT, mR;
      D4* xl;
      Packed* pk;
      std::uint8_t const* ty;
      int const* aatom;
      std::uint16_t* ncnt;
      std::uint16_t* nbr;
      double* v;
      double const* hist;
      std::uint8_t const* mob;
      double* rho0;
      std::uint16_t* need;
      int* mark;
      long long* dacc;
      double rc2;
      float rc2f;
      double L[3], invL[3];
      float Lf[3];
      bool per[3], periodic;
      double shift[3];
      __device__ double* V(int k) const { return v + static_cast<std::int64_t>(k) * M; }
      __device__ double* sT(int j) const { return v + static_cast<std::int64_t>(N_VEC + j) * M; }
      __device__ double* yT(int j) const { return v + static_cast<std::int64_t>(N_VEC + mT + j) * M; }
      __device__ double* sR(int j) const { return v + static_cast<std::int64_t>(N_VEC + 2 * mT + j) * M; }
      __device__ double* yR(int j) const { return v + static_cast<std::int64_t>(N_VEC + 2 * mT + mR + j) * M; }
    };

    __device__ inline double& comp(D4& p, int c) { return c == 0 ? p.x : c == 1 ? p.y : p.z; }

    __device__ inline void pack_one(Ctx const& c, int a) {
      D4 const p = c.xl[a];
      double const X = p.x + c.shift[0], Y = p.y + c.shift[1], Z = p.z + c.shift[2];
      Packed& q = c.pk[a];
      float const hx = static_cast<float>(X), hy = static_cast<float>(Y), hz = static_cast<float>(Z);
      q.hx = hx;
      q.hy = hy;
      q.hz = hz;
      q.lx = static_cast<float>(X - static_cast<double>(hx));
      q.ly = static_cast<float>(Y - static_cast<double>(hy));
      q.lz = static_cast<float>(Z - static_cast<double>(hz));
      q.type = static_cast<std::uint32_t>(c.ty[a]) | (c.mob[a] ? MOBILE_BIT : 0u);
    }

    // ------------------------------------------------------------------ pair geometry

    __device__ inline void dr64(Ctx const& c, int i, int j, double& dx, double& dy, double& dz) {
      D4 const a = c.xl[i], b = c.xl[j];
      dx = b.x - a.x;
      dy = b.y - a.y;
      dz = b.z - a.z;
      if (c.periodic) {
        if (c.per[0]) dx -= c.L[0] * rint(dx * c.invL[0]);
        if (c.per[1]) dy -= c.L[1] * rint(dy * c.invL[1]);
        if (c.per[2]) dz -= c.L[2] * rint(dz * c.invL[2]);
      }
    }

    __device__ inline void dr32(Ctx const& c, Packed const& me, int i, int j, float& dx, float& dy, float& dz) {
      if (c.periodic) {
        double a, b, d;
        dr64(c, i, j, a, b, d);
        dx = static_cast<float>(a);
        dy = static_cast<float>(b);
        dz = static_cast<float>(d);
      } else {
        Packed const o = c.pk[j];
        dx = (o.hx - me.hx) + (o.lx - me.lx);
        dy = (o.hy - me.hy) + (o.ly - me.ly);
        dz = (o.hz - me.hz) + (o.lz - me.lz);
      }
    }

    __device__ inline bool fetch64(double x, double inv_dx, double dx, int n, long long& i, double& x0) {
      if (!(x >= 0)) return false;
      double const u = x * inv_dx;
      if (!(u < static_cast<double>(n))) return false;
      i = static_cast<long long>(u);
      x0 = x - static_cast<double>(i) * dx;
      return true;
    }

    __device__ inline bool fetch32(float r, float inv_dx, int n, int& i, float& t) {
      float const u = r * inv_dx;
      if (!(u >= 0.f) || !(u < static_cast<float>(n))) return false;
      i = static_cast<int>(u);
      t = u - static_cast<float>(i);
      return true;
    }

    template <int LPA>
    __device__ inline double lane_sum(double v) {
#pragma unroll
      for (int o = LPA / 2; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o, LPA);
      return v;
    }

    // ------------------------------------------------------------------ EAM passes (all threads)

    // Density pass over all atoms: F'(rho) into xl[i].w (and pk[i].fp). With ENERGY, accumulates
    // 0.5 * sum v + F(rho) into *e (per thread).
    template <bool MIXED, int LPA, bool ENERGY>
    __device__ void density(Ctx const& c, TablesView const& tb, Blk& sh, double* e) {
      int const nt = blockDim.x;
      int const total = c.n * LPA;
      int const rounds = (total + nt - 1) / nt;
      int const nty = tb.n_types;
      for (int r = 0; r < rounds; ++r) {
        int const t = r * nt + threadIdx.x;
        bool const valid = t < total;
        int const i = valid ? t / LPA : 0;
        int const l = t % LPA;
        double rho = 0, vs = 0;
        if (valid) {
          int const ti = c.ty[i];
          int const cnt = c.ncnt[i];
          if (MIXED) {
            Packed const me = c.pk[i];
            float rf = 0.f, vf = 0.f;
            int chunk = 0;
            for (int k = l; k < cnt; k += LPA) {
              int const j = c.nbr[static_cast<std::int64_t>(k) * c.n + i];
              float dx, dy, dz;
              dr32(c, me, i, j, dx, dy, dz);
              float const r2 = dx * dx + dy * dy + dz * dz;
              if (r2 < c.rc2f) {
                int const tj = c.ty[j];
                int ii;
                float tt;
                if (!fetch32(sqrtf(r2), tb.finv_dR, tb.nR, ii, tt)) {
                  atomicOr(&sh.flag, F_OOB);
                  continue;
                }
                float4 const cp = __ldg(&tb.phi32[static_cast<std::int64_t>(tj + nty * ti) * tb.nR + ii]);
                rf += cp.x + tt * (cp.y + tt * (cp.z + tt * cp.w));
                if (ENERGY) {
                  float4 const cv = __ldg(&tb.v32[static_cast<std::int64_t>(ti + nty * tj) * tb.nR + ii]);
                  vf += cv.x + tt * (cv.y + tt * (cv.z + tt * cv.w));
                }
              }
              if (++chunk == 8) {
                rho += static_cast<double>(rf);
                if (ENERGY) vs += static_cast<double>(vf);
                rf = vf = 0.f;
                chunk = 0;
              }
            }
            rho += static_cast<double>(rf);
            if (ENERGY) vs += static_cast<double>(vf);
          } else {
            for (int k = l; k < cnt; k += LPA) {
              int const j = c.nbr[static_cast<std::int64_t>(k) * c.n + i];
              double dx, dy, dz;
              dr64(c, i, j, dx, dy, dz);
              double const r2 = (dx * dx + dy * dy) + dz * dz;
              if (r2 < c.rc2) {
                int const tj = c.ty[j];
                long long ii;
                double x0;
                if (!fetch64(sqrt(r2), tb.inv_dR, tb.dR, tb.nR, ii, x0)) {
                  atomicOr(&sh.flag, F_OOB);
                  continue;
                }
                D4 const cp = tb.phi64[static_cast<std::int64_t>(tj + nty * ti) * tb.nR + ii];
                rho += cp.x + x0 * (cp.y + x0 * (cp.z + x0 * cp.w));
                if (ENERGY) {
                  D4 const cv = tb.v64[static_cast<std::int64_t>(ti + nty * tj) * tb.nR + ii];
                  vs += cv.x + x0 * (cv.y + x0 * (cv.z + x0 * cv.w));
                }
              }
            }
          }
        }
        rho = lane_sum<LPA>(rho);
        if (ENERGY) vs = lane_sum<LPA>(vs);
        if (valid && l == 0) {
          int const ti = c.ty[i];
          long long ii;
          double x0;
          double fp = 0, fe = 0;
          if (fetch64(rho, tb.inv_dP, tb.dP, tb.nP, ii, x0)) {
            D4 const cf = tb.F64[static_cast<std::int64_t>(ti) * tb.nP + ii];
            fp = cf.y + x0 * (2.0 * cf.z + x0 * 3.0 * cf.w);
            if (ENERGY) fe = cf.x + x0 * (cf.y + x0 * (cf.z + x0 * cf.w));
          } else {
            atomicOr(&sh.flag, F_OOB);
          }
          c.xl[i].w = fp;
          if (MIXED) c.pk[i].fp = static_cast<float>(fp);
          if (ENERGY) *e += 0.5 * vs + fe;
        }
      }
    }

    // Gradient of atom i over its walk (entries k = l, l + step, ...): the reference's pass-2 term
    // (v'(r) + F'_i phi'_{t_j t_i}(r) + F'_j phi'_{t_i t_j}(r)) (r_j - r_i)/r with the sign of a
    // gradient, in groups of U (see rho_walk32). Binary32 terms, binary64 sums of 8 terms; non-periodic.
    __device__ inline bool force_walk32(Ctx const& c, TablesView const& tb, int i, int ti, int l, int step, int cnt,
                                        double& gx, double& gy, double& gz) {
      int const nty = tb.n_types;
      float const inv = tb.finv_dR;
      Packed const me = c.pk[i];
      bool ok = true;
      float fx = 0.f, fy = 0.f, fz = 0.f;
      int grp = 0;
      for (int k = l; k < cnt; k += U * step) {
        int j[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          int const kk = k + u * step;
          j[u] = kk < cnt ? c.nbr[static_cast<std::int64_t>(kk) * c.n + i] : -1;
        }
        Packed o[U];
#pragma unroll
        for (int u = 0; u < U; ++u) o[u] = c.pk[j[u] < 0 ? i : j[u]];
        float dx[U], dy[U], dz[U], ir[U], tt[U];
        std::int64_t rij[U], rji[U];
        bool use[U], same[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          dx[u] = (o[u].hx - me.hx) + (o[u].lx - me.lx);
          dy[u] = (o[u].hy - me.hy) + (o[u].ly - me.ly);
          dz[u] = (o[u].hz - me.hz) + (o[u].lz - me.lz);
          float const r2 = dx[u] * dx[u] + dy[u] * dy[u] + dz[u] * dz[u];
          bool const in = j[u] >= 0 && r2 < c.rc2f;
          ir[u] = rsqrtf(r2);
          float const x = r2 * ir[u] * inv;
          bool const tab = x >= 0.f && x < static_cast<float>(tb.nR);
          ok = ok && (!in || tab);
          use[u] = in && tab;
          int const ii = use[u] ? static_cast<int>(x) : 0;
          tt[u] = x - static_cast<float>(ii);
          int const tj = static_cast<int>(o[u].type & TYPE_MASK);
          same[u] = tj == ti;
          rij[u] = static_cast<std::int64_t>(ti * nty + tj) * tb.nR + ii;  // merged (t_i, t_j) record
          rji[u] = static_cast<std::int64_t>(tj * nty + ti) * tb.nR + ii;  // merged (t_j, t_i) record
        }
        // (t_i, t_j) record: phi_{j->i} and v; phi_{i->j} is the same function for equal types, else the
        // phi of the (t_j, t_i) record
        // (128-bit loads: ptxas of CUDA 13.0 fails on the 256-bit form in the register-capped variant)
        float4 cv[U], ca[U], cb[U];
        float4 const z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < U; ++u) {
          ca[u] = use[u] ? __ldg(&tb.pv32[rij[u]].phi) : z4;
          cv[u] = use[u] ? __ldg(&tb.pv32[rij[u]].v) : z4;
        }
#pragma unroll
        for (int u = 0; u < U; ++u) cb[u] = use[u] && !same[u] ? __ldg(&tb.pv32[rji[u]].phi) : ca[u];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          float const t = tt[u];
          float const dv = cv[u].y + t * (2.f * cv[u].z + 3.f * t * cv[u].w);
          float const da = ca[u].y + t * (2.f * ca[u].z + 3.f * t * ca[u].w);
          float const db = cb[u].y + t * (2.f * cb[u].z + 3.f * t * cb[u].w);
          float const s = use[u] ? (dv + me.fp * da + o[u].fp * db) * inv * ir[u] : 0.f;
          fx -= s * dx[u];
          fy -= s * dy[u];
          fz -= s * dz[u];
        }
        if (++grp == 8 / U) {
          gx += static_cast<double>(fx);
          gy += static_cast<double>(fy);
          gz += static_cast<double>(fz);
          fx = fy = fz = 0.f;
          grp = 0;
        }
      }
      gx += static_cast<double>(fx);
      gy += static_cast<double>(fy);
      gz += static_cast<double>(fz);
      return ok;
    }

    // force_walk32 in binary64 (any box), terms added in walk order.
    __device__ inline bool force_walk64(Ctx const& c, TablesView const& tb, int i, int ti, int l, int step, int cnt,
                                        double& gx, double& gy, double& gz) {
      int const nty = tb.n_types;
      D4 const a = c.xl[i];
      bool ok = true;
      for (int k = l; k < cnt; k += U64 * step) {
        int j[U64];
#pragma unroll
        for (int u = 0; u < U64; ++u) {
          int const kk = k + u * step;
          j[u] = kk < cnt ? c.nbr[static_cast<std::int64_t>(kk) * c.n + i] : -1;
        }
        D4 b[U64];
        int tj[U64];
#pragma unroll
        for (int u = 0; u < U64; ++u) {
          int const jj = j[u] < 0 ? i : j[u];
          b[u] = c.xl[jj];
          tj[u] = c.ty[jj];
        }
        double dx[U64], dy[U64], dz[U64], r[U64], x0[U64];
        std::int64_t rij[U64], rji[U64];
        bool use[U64];
#pragma unroll
        for (int u = 0; u < U64; ++u) {
          dx[u] = b[u].x - a.x;
          dy[u] = b[u].y - a.y;
          dz[u] = b[u].z - a.z;
          if (c.periodic) {
            if (c.per[0]) dx[u] -= c.L[0] * rint(dx[u] * c.invL[0]);
            if (c.per[1]) dy[u] -= c.L[1] * rint(dy[u] * c.invL[1]);
            if (c.per[2]) dz[u] -= c.L[2] * rint(dz[u] * c.invL[2]);
          }
          double const r2 = (dx[u] * dx[u] + dy[u] * dy[u]) + dz[u] * dz[u];
          bool const in = j[u] >= 0 && r2 < c.rc2;
          r[u] = sqrt(r2);
          double const x = r[u] * tb.inv_dR;
          bool const tab = x < static_cast<double>(tb.nR);
          ok = ok && (!in || tab);
          use[u] = in && tab;
          long long const ii = use[u] ? static_cast<long long>(x) : 0;
          x0[u] = r[u] - static_cast<double>(ii) * tb.dR;
          rij[u] = static_cast<std::int64_t>(tj[u] + nty * ti) * tb.nR + ii;
          rji[u] = static_cast<std::int64_t>(ti + nty * tj[u]) * tb.nR + ii;
        }
        D4 cv[U64], ca[U64], cb[U64];
        D4 const z4{0, 0, 0, 0};
#pragma unroll
        for (int u = 0; u < U64; ++u) {
          cv[u] = use[u] ? tb.v64[rij[u]] : z4;
          ca[u] = use[u] ? tb.phi64[rij[u]] : z4;
          cb[u] = use[u] ? tb.phi64[rji[u]] : z4;
        }
#pragma unroll
        for (int u = 0; u < U64; ++u) {
          if (!use[u]) continue;
          double const t = x0[u];
          double const mag = (cv[u].y + t * (2.0 * cv[u].z + t * 3.0 * cv[u].w)) +
                             a.w * (ca[u].y + t * (2.0 * ca[u].z + t * 3.0 * ca[u].w)) +
                             b[u].w * (cb[u].y + t * (2.0 * cb[u].z + t * 3.0 * cb[u].w));
          double const s = mag / r[u];
          gx -= s * dx[u];
          gy -= s * dy[u];
          gz -= s * dz[u];
        }
      }
      return ok;
    }

    // Force pass over mobile atoms into out (3 per mobile atom).
    template <bool MIXED, int LPA>
    __device__ void force(Ctx const& c, TablesView const& tb, Blk& sh, typename std::conditional<MIXED, float, double>::type* out) {
      int const nt = blockDim.x;
      int const total = c.na * LPA;
      int const rounds = (total + nt - 1) / nt;
      int const nty = tb.n_types;
      for (int r = 0; r < rounds; ++r) {
        int const t = r * nt + threadIdx.x;
        bool const valid = t < total;
        int const k0 = valid ? t / LPA : 0;
        int const l = t % LPA;
        int const i = valid ? c.aatom[k0] : 0;
        double gx = 0, gy = 0, gz = 0;
        if (valid) {
          int const ti = c.ty[i];
          int const cnt = c.ncnt[i];
          if (!MIXED) {
            if (!force_walk64(c, tb, i, ti, l, LPA, cnt, gx, gy, gz)) atomicOr(&sh.flag, F_OOB);
          } else if (!c.periodic) {
            if (!force_walk32(c, tb, i, ti, l, LPA, cnt, gx, gy, gz)) atomicOr(&sh.flag, F_OOB);
          } else {  // periodic boxes: binary32 differences of the binary64 minimum images
            Packed const me = c.pk[i];
            float fx = 0.f, fy = 0.f, fz = 0.f;
            int chunk = 0;
            float const inv = tb.finv_dR;
            for (int k = l; k < cnt; k += LPA) {
              int const j = c.nbr[static_cast<std::int64_t>(k) * c.n + i];
              float dx, dy, dz;
              dr32(c, me, i, j, dx, dy, dz);
              float const r2 = dx * dx + dy * dy + dz * dz;
              if (r2 < c.rc2f) {
                float const ir = rsqrtf(r2);
                int const tj = c.ty[j];
                int ii;
                float tt;
                if (!fetch32(r2 * ir, inv, tb.nR, ii, tt)) {
                  atomicOr(&sh.flag, F_OOB);
                  continue;
                }
                float4 const cv = __ldg(&tb.v32[static_cast<std::int64_t>(tj + nty * ti) * tb.nR + ii]);
                float4 const ca = __ldg(&tb.phi32[static_cast<std::int64_t>(tj + nty * ti) * tb.nR + ii]);
                float4 const cb = __ldg(&tb.phi32[static_cast<std::int64_t>(ti + nty * tj) * tb.nR + ii]);
                float const dv = cv.y + tt * (2.f * cv.z + 3.f * tt * cv.w);
                float const da = ca.y + tt * (2.f * ca.z + 3.f * tt * ca.w);
                float const db = cb.y + tt * (2.f * cb.z + 3.f * tt * cb.w);
                float const fpj = c.pk[j].fp;
                float const s = (dv + me.fp * da + fpj * db) * inv * ir;
                fx -= s * dx;
                fy -= s * dy;
                fz -= s * dz;
              }
              if (++chunk == 8) {
                gx += static_cast<double>(fx);
                gy += static_cast<double>(fy);
                gz += static_cast<double>(fz);
                fx = fy = fz = 0.f;
                chunk = 0;
              }
            }
            gx += static_cast<double>(fx);
            gy += static_cast<double>(fy);
            gz += static_cast<double>(fz);
          }
        }
        gx = lane_sum<LPA>(gx);
        gy = lane_sum<LPA>(gy);
        gz = lane_sum<LPA>(gz);
        if (valid && l == 0) {
          using O = typename std::conditional<MIXED, float, double>::type;
          out[3 * k0 + 0] = static_cast<O>(gx);
          out[3 * k0 + 1] = static_cast<O>(gy);
          out[3 * k0 + 2] = static_cast<O>(gz);
        }
      }
    }

    // Pair density term phi(t_j, t_i)(r_ij) of neighbour j at atom i: binary32 (MIXED) or binary64.
    template <bool MIXED>
    __device__ inline bool rho_term(Ctx const& c, TablesView const& tb, Packed const& me, int i, int ti, int j,
                                    float& rf, double& rd) {
      int const nty = tb.n_types;
      if (MIXED) {
        float dx, dy, dz;
        dr32(c, me, i, j, dx, dy, dz);
        float const r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < c.rc2f) {
          int ii;
          float tt;
          if (!fetch32(sqrtf(r2), tb.finv_dR, tb.nR, ii, tt)) return false;
          float4 const cp = __ldg(&tb.phi32[static_cast<std::int64_t>(c.ty[j] + nty * ti) * tb.nR + ii]);
          rf += cp.x + tt * (cp.y + tt * (cp.z + tt * cp.w));
        }
      } else {
        double dx, dy, dz;
        dr64(c, i, j, dx, dy, dz);
        double const r2 = (dx * dx + dy * dy) + dz * dz;
        if (r2 < c.rc2) {
          long long ii;
          double x0;
          if (!fetch64(sqrt(r2), tb.inv_dR, tb.dR, tb.nR, ii, x0)) return false;
          D4 const cp = tb.phi64[static_cast<std::int64_t>(c.ty[j] + nty * ti) * tb.nR + ii];
          rd += cp.x + x0 * (cp.y + x0 * (cp.z + x0 * cp.w));
        }
      }
      return true;
    }

    // ------------------------------------------------------------------ grouped neighbour walks
    //
    // The gradient's pair loops walk one atom's list column (entries k = l, l + step, ... < cnt) in
    // groups of U: the list entries, slot records and spline rows of a group are all loaded before any
    // is used, so a lane keeps U independent gather chains in flight. The search kernel runs a few warps
    // per SM, and one entry-record-row chain costs hundreds of cycles, so this is what bounds a pass.
    // Missing entries of the last group read the atom's own record and are masked out. (U is defined
    // at the top of the file.)

    // Density walk of mobile atom i: returns in rho the sum of phi(t_j, t_i)(r_ij) over the walk and
    // adds phi(t_i, t_j)(r_ij) to the accumulator of every static neighbour j (fixed point, L2 atomics),
    // so a static atom's density is its fixed static part plus one accumulator read. Binary32 terms,
    // binary64 sums of 8 terms; non-periodic boxes. False when a distance fell outside the table.
    __device__ inline bool rho_walk32(Ctx const& c, TablesView const& tb, int i, int ti, Packed const& me, int l,
                                      int step, int cnt, double& rho) {
      int const nty = tb.n_types;
      float const sc = static_cast<float>(dacc_scale<true>());
      bool ok = true;
      float rf = 0.f;
      int grp = 0;
      for (int k = l; k < cnt; k += U * step) {
        int j[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          int const kk = k + u * step;
          j[u] = kk < cnt ? c.nbr[static_cast<std::int64_t>(kk) * c.n + i] : -1;
        }
        Packed o[U];
#pragma unroll
        for (int u = 0; u < U; ++u) o[u] = c.pk[j[u] < 0 ? i : j[u]];
        float tt[U];
        std::int64_t rown[U], rowo[U];
        bool use[U], stat[U], same[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          float const dx = (o[u].hx - me.hx) + (o[u].lx - me.lx);
          float const dy = (o[u].hy - me.hy) + (o[u].ly - me.ly);
          float const dz = (o[u].hz - me.hz) + (o[u].lz - me.lz);
          float const r2 = dx * dx + dy * dy + dz * dz;
          bool const in = j[u] >= 0 && r2 < c.rc2f;
          float const x = sqrtf(r2) * tb.finv_dR;
          bool const tab = x < static_cast<float>(tb.nR);
          ok = ok && (!in || tab);
          use[u] = in && tab;
          stat[u] = use[u] && (o[u].type & MOBILE_BIT) == 0;
          int const ii = use[u] ? static_cast<int>(x) : 0;
          tt[u] = x - static_cast<float>(ii);
          int const tj = static_cast<int>(o[u].type & TYPE_MASK);
          same[u] = tj == ti;
          rown[u] = static_cast<std::int64_t>(ti * nty + tj) * tb.nR + ii;  // merged (t_i, t_j): phi_{j->i}
          rowo[u] = static_cast<std::int64_t>(tj * nty + ti) * tb.nR + ii;  // merged (t_j, t_i): phi_{i->j}
        }
        float4 cp[U], cq[U];
        float4 const z4 = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
        for (int u = 0; u < U; ++u) cp[u] = use[u] ? __ldg(&tb.pv32[rown[u]].phi) : z4;
#pragma unroll
        for (int u = 0; u < U; ++u) cq[u] = stat[u] && !same[u] ? __ldg(&tb.pv32[rowo[u]].phi) : cp[u];
#pragma unroll
        for (int u = 0; u < U; ++u) {
          float const t = tt[u];
          rf += cp[u].x + t * (cp[u].y + t * (cp[u].z + t * cp[u].w));
          if (stat[u]) {
            float const q = cq[u].x + t * (cq[u].y + t * (cq[u].z + t * cq[u].w));
            atomicAdd(reinterpret_cast<unsigned long long*>(c.dacc + j[u]),
                      static_cast<unsigned long long>(__float2ll_rn(q * sc)));
          }
        }
        if (++grp == 8 / U) {
          rho += static_cast<double>(rf);
          rf = 0.f;
          grp = 0;
        }
      }
      rho += static_cast<double>(rf);
      return ok;
    }

    // rho_walk32 in binary64 (any box); own terms added in walk order.
    __device__ inline bool rho_walk64(Ctx const& c, TablesView const& tb, int i, int ti, int l, int step, int cnt,
                                      double& rho) {
      int const nty = tb.n_types;
      double const sc = dacc_scale<false>();
      bool ok = true;
      D4 const a = c.xl[i];
      for (int k = l; k < cnt; k += U64 * step) {
        int j[U64];
#pragma unroll
        for (int u = 0; u < U64; ++u) {
          int const kk = k + u * step;
          j[u] = kk < cnt ? c.nbr[static_cast<std::int64_t>(kk) * c.n + i] : -1;
        }
        D4 b[U64];
        int tj[U64];
        bool mj[U64];
#pragma unroll
        for (int u = 0; u < U64; ++u) {
          int const jj = j[u] < 0 ? i : j[u];
          b[u] = c.xl[jj];
          tj[u] = c.ty[jj];
          mj[u] = c.mob[jj] != 0;
        }
        double x0[U64];
        std::int64_t rown[U64], rowo[U64];
        bool use[U64], stat[U64];
#pragma unroll
        for (int u = 0; u < U64; ++u) {
          double dx = b[u].x - a.x, dy = b[u].y - a.y, dz = b[u].z - a.z;
          if (c.periodic) {
            if (c.per[0]) dx -= c.L[0] * rint(dx * c.invL[0]);
            if (c.per[1]) dy -= c.L[1] * rint(dy * c.invL[1]);
            if (c.per[2]) dz -= c.L[2] * rint(dz * c.invL[2]);
          }
          double const r2 = (dx * dx + dy * dy) + dz * dz;
          bool const in = j[u] >= 0 && r2 < c.rc2;
          double const r = sqrt(r2);
          double const x = r * tb.inv_dR;
          bool const tab = x < static_cast<double>(tb.nR);
          ok = ok && (!in || tab);
          use[u] = in && tab;
          stat[u] = use[u] && !mj[u];
          long long const ii = use[u] ? static_cast<long long>(x) : 0;
          x0[u] = r - static_cast<double>(ii) * tb.dR;
          rown[u] = static_cast<std::int64_t>(tj[u] + nty * ti) * tb.nR + ii;
          rowo[u] = static_cast<std::int64_t>(ti + nty * tj[u]) * tb.nR + ii;
        }
        D4 cp[U64], cq[U64];
        D4 const z4{0, 0, 0, 0};
#pragma unroll
        for (int u = 0; u < U64; ++u) {
          cp[u] = use[u] ? tb.phi64[rown[u]] : z4;
          cq[u] = stat[u] ? tb.phi64[rowo[u]] : z4;
        }
#pragma unroll
        for (int u = 0; u < U64; ++u) {
          double const t = x0[u];
          if (use[u]) rho += cp[u].x + t * (cp[u].y + t * (cp[u].z + t * cp[u].w));
          if (stat[u]) {
            double const q = cq[u].x + t * (cq[u].y + t * (cq[u].z + t * cq[u].w));
            atomicAdd(reinterpret_cast<unsigned long long*>(c.dacc + j[u]),
                      static_cast<unsigned long long>(__double2ll_rn(q * sc)));
          }
        }
      }
      return ok;
    }

    // The same walk for periodic binary32-pair searches (minimum images in binary64), one entry at a time.
    __device__ inline bool rho_walk32_periodic(Ctx const& c, TablesView const& tb, int i, int ti, Packed const& me,
                                               int l, int step, int cnt, double& rho) {
      int const nty = tb.n_types;
      float const sc = static_cast<float>(dacc_scale<true>());
      bool ok = true;
      float rf = 0.f;
      int chunk = 0;
      for (int k = l; k < cnt; k += step) {
        int const j = c.nbr[static_cast<std::int64_t>(k) * c.n + i];
        float dx, dy, dz;
        dr32(c, me, i, j, dx, dy, dz);
        float const r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < c.rc2f) {
          int ii;
          float tt;
          if (!fetch32(sqrtf(r2), tb.finv_dR, tb.nR, ii, tt)) {
            ok = false;
          } else {
            int const tj = c.ty[j];
            float4 const cp = __ldg(&tb.phi32[static_cast<std::int64_t>(tj + nty * ti) * tb.nR + ii]);
            rf += cp.x + tt * (cp.y + tt * (cp.z + tt * cp.w));
            if (!c.mob[j]) {
              float4 const cq = __ldg(&tb.phi32[static_cast<std::int64_t>(ti + nty * tj) * tb.nR + ii]);
              float const q = cq.x + tt * (cq.y + tt * (cq.z + tt * cq.w));
              atomicAdd(reinterpret_cast<unsigned long long*>(c.dacc + j),
                        static_cast<unsigned long long>(__float2ll_rn(q * sc)));
            }
          }
        }
        if (++chunk == 8) {
          rho += static_cast<double>(rf);
          rf = 0.f;
          chunk = 0;
        }
      }
      rho += static_cast<double>(rf);
      return ok;
    }

    // Density of every static atom from its static neighbours. Static atoms never move during a
    // search, so this part of their density is fixed; computed once per search (all threads).
    template <bool MIXED>
    __device__ void static_density(Ctx const& c, TablesView const& tb, Blk& sh) {
      for (int b = threadIdx.x; b < c.n; b += blockDim.x) {
        if (c.mob[b]) continue;
        Packed const me = c.pk[b];
        int const tb_ = c.ty[b];
        double rho = 0;
        float rf = 0.f;
        int const cnt = c.ncnt[b];
        for (int k = 0; k < cnt; ++k) {
          int const j = c.nbr[static_cast<std::int64_t>(k) * c.n + b];
          if (c.mob[j]) continue;
          if (!rho_term<MIXED>(c, tb, me, b, tb_, j, rf, rho)) atomicOr(&sh.flag, F_OOB);
          if (MIXED && (k & 7) == 7) {
            rho += static_cast<double>(rf);
            rf = 0.f;
          }
        }
        c.rho0[b] = rho + static_cast<double>(rf);
      }
    }

    // F'(rho) of atom i (embedding spline, binary64) into xl[i].w and, for binary32 pairs, pk[i].fp.
    template <bool MIXED>
    __device__ inline void store_fprime(Ctx const& c, TablesView const& tb, Blk& sh, int i, double rho) {
      long long ii;
      double x0;
      double fp = 0;
      if (fetch64(rho, tb.inv_dP, tb.dP, tb.nP, ii, x0)) {
        D4 const cf = tb.F64[static_cast<std::int64_t>(c.ty[i]) * tb.nP + ii];
        fp = cf.y + x0 * (2.0 * cf.z + x0 * 3.0 * cf.w);
      } else {
        atomicOr(&sh.flag, F_OOB);
      }
      c.xl[i].w = fp;
      if (MIXED) c.pk[i].fp = static_cast<float>(fp);
    }

    // Density pass of one gradient evaluation over the atoms whose F' the force pass reads. Each mobile
    // atom walks all its neighbours with a group of W lanes (its own density) and scatters its terms to
    // its static neighbours' accumulators; then each needed static atom takes its fixed static density
    // plus its accumulator (read and cleared in one exchange).
    template <bool MIXED, int W>
    __device__ void density_inc(Ctx const& c, TablesView const& tb, Blk& sh) {
      int const nt = blockDim.x;
      int const nm = c.na * W;
      int const rounds = (nm + nt - 1) / nt;
      for (int r = 0; r < rounds; ++r) {
        int const t = r * nt + threadIdx.x;
        bool const valid = t < nm;
        int const i = valid ? c.aatom[t / W] : 0;
        int const l = t % W;
        double rho = 0;
        if (valid) {
          int const ti = c.ty[i];
          int const cnt = c.ncnt[i];
          bool ok;
          if (!MIXED) {
            ok = rho_walk64(c, tb, i, ti, l, W, cnt, rho);
          } else if (!c.periodic) {
            ok = rho_walk32(c, tb, i, ti, c.pk[i], l, W, cnt, rho);
          } else {
            ok = rho_walk32_periodic(c, tb, i, ti, c.pk[i], l, W, cnt, rho);
          }
          if (!ok) atomicOr(&sh.flag, F_OOB);
        }
        rho = lane_sum<W>(rho);
        if (valid && l == 0) store_fprime<MIXED>(c, tb, sh, i, rho);
      }
      __syncthreads();
      double const inv = 1.0 / dacc_scale<MIXED>();
      for (int q = threadIdx.x; q < sh.n_need; q += nt) {
        int const b = c.need[q];
        long long const a = static_cast<long long>(atomicExch(reinterpret_cast<unsigned long long*>(c.dacc + b), 0ull));
        store_fprime<MIXED>(c, tb, sh, b, c.rho0[b] + static_cast<double>(a) * inv);
      }
    }

    // Lanes per mobile atom in the EAM passes: the widest power of two (at least LPA, at most 32) that
    // keeps the mobile atoms within one round of the block.
    template <int LPA>
    __device__ inline int wide_lanes(int na) {
      int w = 32;
      while (w > LPA && na * w > static_cast<int>(blockDim.x)) w >>= 1;
      return w;
    }

    template <bool MIXED, int W>
    __device__ void passes(Ctx const& c, TablesView const& tb, Blk& sh, typename std::conditional<MIXED, float, double>::type* out) {
      density_inc<MIXED, W>(c, tb, sh);
      __syncthreads();
      force<MIXED, W>(c, tb, sh, out);
    }

    // One EAM gradient evaluation into out (mobile DOFs). Called by every thread; returns true when a
    // device-side error was raised (the caller ends the search).
    template <bool MIXED, int LPA>
    __device__ bool gradient(Ctx const& c, TablesView const& tb, Blk& sh, typename std::conditional<MIXED, float, double>::type* out) {
      __syncthreads();
      if (MIXED) {
        for (int k = threadIdx.x; k < c.na; k += blockDim.x) pack_one(c, c.aatom[k]);
        __syncthreads();
      }
      switch (wide_lanes<LPA>(c.na)) {
        case 32: passes<MIXED, 32>(c, tb, sh, out); break;
        case 16: passes<MIXED, 16>(c, tb, sh, out); break;
        case 8: passes<MIXED, (LPA > 8 ? LPA : 8)>(c, tb, sh, out); break;
        case 4: passes<MIXED, (LPA > 4 ? LPA : 4)>(c, tb, sh, out); break;
        case 2: passes<MIXED, (LPA > 2 ? LPA : 2)>(c, tb, sh, out); break;
        default: passes<MIXED, LPA>(c, tb, sh, out); break;
      }
      __syncthreads();
      int const f = sh.flag;
      if (threadIdx.x == 0) c.S->grad_calls += 1;
      return f != 0;
    }

    template <bool MIXED, int LPA>
    __device__ double energy(Ctx const& c, TablesView const& tb, Blk& sh) {
      __syncthreads();
      if (MIXED) {
        for (int k = threadIdx.x; k < c.na; k += blockDim.x) pack_one(c, c.aatom[k]);
        __syncthreads();
      }
      double e = 0.0;
      density<MIXED, LPA, true>(c, tb, sh, &e);
      return block_sum(e, sh);
    }

    // ------------------------------------------------------------------ neighbour list (all threads)

    // List::rebuild (list.cpp:53-95): canonical images of the mobile positions, then every pair within
    // rc_list (plus a margin covering binary32 rounding) -- a superset of the reference's list, so the
    // exact r < r_cut filter at evaluation time sees the same pairs. Returns true on error.
    __device__ void static_lists(Ctx const& c, Blk& sh, double rc_list);

    __device__ bool rebuild(Ctx const& c, Blk& sh, double rc_list) {
      __syncthreads();
      double const* X = c.V(V_X);
      for (int e = threadIdx.x; e < c.M; e += blockDim.x) {
        int const k = e % 3;
        comp(c.xl[c.aatom[e / 3]], k) = X[e] - c.L[k] * floor(X[e] * c.invL[k]);
      }
      __syncthreads();
      for (int k = threadIdx.x; k < c.na; k += blockDim.x) pack_one(c, c.aatom[k]);
      __syncthreads();
      float const lim = static_cast<float>((rc_list + 1e-3) * (rc_list + 1e-3));
      for (int i = threadIdx.x; i < c.n; i += blockDim.x) {
        Packed const me = c.pk[i];
        int cnt = 0;
        for (int j = 0; j < c.n; ++j) {
          Packed const o = c.pk[j];
          float dx = o.hx - me.hx, dy = o.hy - me.hy, dz = o.hz - me.hz;
          if (c.periodic) {
            if (c.per[0]) dx -= c.Lf[0] * rintf(dx / c.Lf[0]);
            if (c.per[1]) dy -= c.Lf[1] * rintf(dy / c.Lf[1]);
            if (c.per[2]) dz -= c.Lf[2] * rintf(dz / c.Lf[2]);
          }
          if (j != i && dx * dx + dy * dy + dz * dz < lim) {
            if (cnt < NB_CAP) c.nbr[static_cast<std::int64_t>(cnt) * c.n + i] = static_cast<std::uint16_t>(j);
            ++cnt;
          }
        }
        if (cnt > NB_CAP) atomicOr(&sh.flag, F_NLIST);
        c.ncnt[i] = static_cast<std::uint16_t>(min(cnt, NB_CAP));
      }
      static_lists(c, sh, rc_list);
      return sh.flag != 0;
    }

    // Static atoms with a mobile neighbour ("needed": the density pass scatters into them and the force
    // pass reads their F'): the static entries of the mobile atoms' lists, which are exactly the static
    // atoms that list a mobile atom (lists are symmetric). The order of the needed list does not matter.
    __device__ void static_lists(Ctx const& c, Blk& sh, double) {
      if (threadIdx.x == 0) sh.n_need = 0;
      for (int b = threadIdx.x; b < c.n; b += blockDim.x) c.mark[b] = 0;
      __syncthreads();
      int const lane = threadIdx.x & 31, nw = blockDim.x >> 5;
      for (int k = threadIdx.x >> 5; k < c.na; k += nw) {
        int const i = c.aatom[k];
        int const cnt = c.ncnt[i];
        for (int e = lane; e < cnt; e += 32) {
          int const j = c.nbr[static_cast<std::int64_t>(e) * c.n + i];
          if (!c.mob[j] && atomicCAS(&c.mark[j], 0, 1) == 0) c.need[atomicAdd(&sh.n_need, 1)] = static_cast<std::uint16_t>(j);
        }
      }
      __syncthreads();
    }

    // Rebuild after a translation step: static atoms never move, so static-static pairs never change.
    // Only the mobile atoms' lists (one warp per mobile atom, in atom order) and the static atoms'
    // mobile-neighbour lists are rebuilt. Returns true on error.
    __device__ bool rebuild_mobile(Ctx const& c, Blk& sh, double rc_list) {
      __syncthreads();
      double const* X = c.V(V_X);
      for (int e = threadIdx.x; e < c.M; e += blockDim.x) {
        int const k = e % 3;
        comp(c.xl[c.aatom[e / 3]], k) = X[e] - c.L[k] * floor(X[e] * c.invL[k]);
      }
      __syncthreads();
      for (int k = threadIdx.x; k < c.na; k += blockDim.x) pack_one(c, c.aatom[k]);
      __syncthreads();
      float const lim = static_cast<float>((rc_list + 1e-3) * (rc_list + 1e-3));
      int const lane = threadIdx.x & 31, nw = blockDim.x >> 5;
      for (int k = threadIdx.x >> 5; k < c.na; k += nw) {
        int const i = c.aatom[k];
        Packed const me = c.pk[i];
        int cnt = 0;
        for (int j0 = 0; j0 < c.n; j0 += 32) {
          int const j = j0 + lane;
          bool hit = false;
          if (j < c.n && j != i) {
            Packed const o = c.pk[j];
            float dx = o.hx - me.hx, dy = o.hy - me.hy, dz = o.hz - me.hz;
            if (c.periodic) {
              if (c.per[0]) dx -= c.Lf[0] * rintf(dx / c.Lf[0]);
              if (c.per[1]) dy -= c.Lf[1] * rintf(dy / c.Lf[1]);
              if (c.per[2]) dz -= c.Lf[2] * rintf(dz / c.Lf[2]);
            }
            hit = dx * dx + dy * dy + dz * dz < lim;
          }
          unsigned const mask = __ballot_sync(FULL, hit);
          if (hit) {
            int const p = cnt + __popc(mask & ((1u << lane) - 1u));
            if (p < NB_CAP) c.nbr[static_cast<std::int64_t>(p) * c.n + i] = static_cast<std::uint16_t>(j);
          }
          cnt += __popc(mask);
        }
        if (lane == 0) {
          if (cnt > NB_CAP) atomicOr(&sh.flag, F_NLIST);
          c.ncnt[i] = static_cast<std::uint16_t>(min(cnt, NB_CAP));
        }
      }
      __syncthreads();
      static_lists(c, sh, rc_list);
      return sh.flag != 0;
    }

    // ------------------------------------------------------------------ warp-0 vector algebra

    // Reductions of the search's vector algebra (warp 0). Binary64 searches sum in binary64. Binary32-pair
    // searches form the per-lane terms and the warp reduction in binary32, and their scalar divisions and
    // square roots are binary32: a dependent binary64 add or multiply costs ~67 cycles on GB300 and a
    // binary64 division or square root hundreds, a binary32 one a few. Positions, gradients and their
    // differences stay binary64; the binary32 sums feed L-BFGS directions, rotation planes, curvatures
    // and convergence tests whose tolerances are orders of magnitude above binary32 rounding.
    template <bool MIXED>
    using Red = typename std::conditional<MIXED, float, double>::type;

    // Storage of a search's per-DOF vectors other than positions: binary32 in binary32-pair searches
    // (a vector keeps its M-double slot and uses the first half of it), binary64 otherwise. Positions
    // (V_X, V_INMIN, the translation L-BFGS's previous x) are binary64 in both.
    template <bool MIXED>
    using Vt = typename std::conditional<MIXED, float, double>::type;

    template <bool MIXED>
    __device__ inline Vt<MIXED>* vp(double* slot) {
      return reinterpret_cast<Vt<MIXED>*>(slot);
    }

    template <bool MIXED>
    __device__ inline Red<MIXED> wsum(Red<MIXED> v) {
      for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
      return v;
    }

    template <bool MIXED, typename A, typename B>
    __device__ inline Red<MIXED> wdot(A const* a, B const* b, int M) {
      Red<MIXED> s = 0;
      for (int e = threadIdx.x; e < M; e += 32) s += static_cast<Red<MIXED>>(a[e]) * static_cast<Red<MIXED>>(b[e]);
      return wsum<MIXED>(s);
    }

    // A scalar of the search algebra: f32() in binary32 on every lane of a binary32-pair search, f64() in
    // binary64 on lane 0 (broadcast) otherwise.
    template <bool MIXED, typename F32, typename F64>
    __device__ inline double scal(F32&& f32, F64&& f64) {
      if constexpr (MIXED) {
        return static_cast<double>(f32());
      } else {
        return lane0(f64);
      }
    }

    // List::update (list.cpp:37-51) on mobile atoms: xl -= d (warp 0).
    template <typename T>
    __device__ inline void wlist_update(Ctx const& c, T const* d, double sign) {
      for (int e = threadIdx.x; e < c.M; e += 32) comp(c.xl[c.aatom[e / 3]], e % 3) -= sign * static_cast<double>(d[e]);
    }

    // The same step with the direction q held in registers (K elements a lane, M <= 32 K): the two-loop
    // recursion is a chain of 2m dependent warp reductions, and this form keeps every memory access off
    // that chain. The next history pair is loaded while the current reduction runs. Each lane sums its
    // elements in the memory form's order, so the results are the same.
    template <bool MIXED, typename XT, int K>
    __device__ __noinline__ void newton_reg(Ctx const& c, int m, int& k, double* s0, double* y0, double* rho, double* alpha,
                               XT* px, Vt<MIXED>* pg, XT const* x, Vt<MIXED> const* g, Vt<MIXED>* out) {
      using R = Red<MIXED>;
      using V = Vt<MIXED>;
      int const M = c.M;
      int const lane = threadIdx.x;
      auto S_ = [&](int j) { return vp<MIXED>(s0 + static_cast<std::int64_t>(j) * M); };
      auto Y_ = [&](int j) { return vp<MIXED>(y0 + static_cast<std::int64_t>(j) * M); };
      int const prev = k > 0 ? (k - 1) % m : 0;
      V q[K];
      if (k > 0) {
        V* sp = S_(prev);
        V* yp = Y_(prev);
        R d = 0;
#pragma unroll
        for (int u = 0; u < K; ++u) {
          int const e = lane + 32 * u;
          if (e < M) {
            V const sv = static_cast<V>(x[e] - px[e]);
            V const yv = g[e] - pg[e];
            sp[e] = sv;
            yp[e] = yv;
            d += static_cast<R>(sv) * static_cast<R>(yv);
          }
        }
        R const ds = wsum<MIXED>(d);
        double const r = scal<MIXED>([&] { return 1.f / fabsf(static_cast<float>(ds)); },
                                     [&] { return 1.0 / fabs(ds); });
        if (lane == 0) rho[prev] = r;
      }
#pragma unroll
      for (int u = 0; u < K; ++u) {
        int const e = lane + 32 * u;
        q[u] = 0;
        if (e < M) {
          px[e] = x[e];
          pg[e] = g[e];
          q[u] = g[e];
        }
      }
      __syncwarp();
      int const incur = k <= m ? 0 : k - m;
      int const bound = k <= m ? k : m;
      auto load = [&](V const* p, V* r) {
#pragma unroll
        for (int u = 0; u < K; ++u) {
          int const e = lane + 32 * u;
          r[u] = e < M ? p[e] : V(0);
        }
      };
      V sv[K], yv[K];
      if (bound > 0) {
        int const j = (bound - 1 + incur) % m;
        load(S_(j), sv);
        load(Y_(j), yv);
      }
      for (int i = bound - 1; i >= 0; --i) {
        int const j = (i + incur) % m;
        V sn[K], yn[K];
        if (i > 0) {
          int const jn = (i - 1 + incur) % m;
          load(S_(jn), sn);
          load(Y_(jn), yn);
        }
        R a = 0;
#pragma unroll
        for (int u = 0; u < K; ++u)
          if (lane + 32 * u < M) a += static_cast<R>(sv[u]) * static_cast<R>(q[u]);
        a = static_cast<R>(rho[j]) * wsum<MIXED>(a);
        if (lane == 0) alpha[j] = a;
        V const av = static_cast<V>(a);
#pragma unroll
        for (int u = 0; u < K; ++u) q[u] -= av * yv[u];
        if (i > 0) {
#pragma unroll
          for (int u = 0; u < K; ++u) {
            sv[u] = sn[u];
            yv[u] = yn[u];
          }
        }
      }
      if (k > 0) {
        V yl[K];
        load(Y_(prev), yl);
        R yy = 0;
#pragma unroll
        for (int u = 0; u < K; ++u)
          if (lane + 32 * u < M) yy += static_cast<R>(yl[u]) * static_cast<R>(yl[u]);
        yy = wsum<MIXED>(yy);
        R const rp = static_cast<R>(rho[prev]);
        V const scale = static_cast<V>(scal<MIXED>([&] { return 1.f / static_cast<float>(rp) / static_cast<float>(yy); },
                                                   [&] { return 1.0 / rp / yy; }));
#pragma unroll
        for (int u = 0; u < K; ++u) q[u] = q[u] * scale;
      }
      __syncwarp();
      if (bound > 0) {
        int const j = incur % m;
        load(S_(j), sv);
        load(Y_(j), yv);
      }
      for (int i = 0; i <= bound - 1; ++i) {
        int const j = (i + incur) % m;
        V sn[K], yn[K];
        if (i < bound - 1) {
          int const jn = (i + 1 + incur) % m;
          load(S_(jn), sn);
          load(Y_(jn), yn);
        }
        R beta = 0;
#pragma unroll
        for (int u = 0; u < K; ++u)
          if (lane + 32 * u < M) beta += static_cast<R>(yv[u]) * static_cast<R>(q[u]);
        beta = static_cast<R>(rho[j]) * wsum<MIXED>(beta);
        V const ab = static_cast<V>(static_cast<R>(alpha[j]) - beta);
#pragma unroll
        for (int u = 0; u < K; ++u) q[u] += ab * sv[u];
        if (i < bound - 1) {
#pragma unroll
          for (int u = 0; u < K; ++u) {
            sv[u] = sn[u];
            yv[u] = yn[u];
          }
        }
      }
#pragma unroll
      for (int u = 0; u < K; ++u) {
        int const e = lane + 32 * u;
        if (e < M) out[e] = q[u];
      }
      __syncwarp();
      ++k;
    }

    // StepLBFGS::newton_step_impl (lbfgs_core.cpp:29-87), warp 0. History slot j of s (y) starts at
    // s0 + j M (y0 + j M) doubles and holds a V vector. x / px are positions (binary64) for the
    // translation and the axis (V) for the rotation. Up to 256 degrees of freedom the direction stays in
    // registers (newton_reg); larger searches keep it in memory.
    template <bool MIXED, typename XT>
    __device__ void newton(Ctx const& c, int m, int& k, double* s0, double* y0, double* rho, double* alpha,
                           XT* px, Vt<MIXED>* pg, XT const* x, Vt<MIXED> const* g, Vt<MIXED>* out) {
      using R = Red<MIXED>;
      using V = Vt<MIXED>;
      int const M = c.M;
      if (M <= 64) return newton_reg<MIXED, XT, 2>(c, m, k, s0, y0, rho, alpha, px, pg, x, g, out);
      if (M <= 128) return newton_reg<MIXED, XT, 4>(c, m, k, s0, y0, rho, alpha, px, pg, x, g, out);
      if (M <= 256) return newton_reg<MIXED, XT, 8>(c, m, k, s0, y0, rho, alpha, px, pg, x, g, out);
      int const lane = threadIdx.x;
      auto S_ = [&](int j) { return vp<MIXED>(s0 + static_cast<std::int64_t>(j) * M); };
      auto Y_ = [&](int j) { return vp<MIXED>(y0 + static_cast<std::int64_t>(j) * M); };
      int const prev = k > 0 ? (k - 1) % m : 0;
      if (k > 0) {
        V* sp = S_(prev);
        V* yp = Y_(prev);
        R d = 0;
        for (int e = lane; e < M; e += 32) {
          sp[e] = static_cast<V>(x[e] - px[e]);
          yp[e] = g[e] - pg[e];
          d += static_cast<R>(sp[e]) * static_cast<R>(yp[e]);
        }
        R const ds = wsum<MIXED>(d);
        double const r = scal<MIXED>([&] { return 1.f / fabsf(static_cast<float>(ds)); },
                                     [&] { return 1.0 / fabs(ds); });
        if (lane == 0) rho[prev] = r;
      }
      for (int e = lane; e < M; e += 32) {
        px[e] = x[e];
        pg[e] = g[e];
        out[e] = g[e];
      }
      __syncwarp();
      int const incur = k <= m ? 0 : k - m;
      int const bound = k <= m ? k : m;
      for (int i = bound - 1; i >= 0; --i) {
        int const j = (i + incur) % m;
        V const* s = S_(j);
        V const* y = Y_(j);
        R const a = static_cast<R>(rho[j]) * wdot<MIXED>(s, out, M);
        if (lane == 0) alpha[j] = a;
        V const av = static_cast<V>(a);
        for (int e = lane; e < M; e += 32) out[e] -= av * y[e];
      }
      if (k > 0) {
        V const* yp = Y_(prev);
        R const yy = wdot<MIXED>(yp, yp, M);
        R const rp = static_cast<R>(rho[prev]);
        V const scale = static_cast<V>(scal<MIXED>([&] { return 1.f / static_cast<float>(rp) / static_cast<float>(yy); },
                                                   [&] { return 1.0 / rp / yy; }));
        for (int e = lane; e < M; e += 32) out[e] = out[e] * scale;
      }
      __syncwarp();
      for (int i = 0; i <= bound - 1; ++i) {
        int const j = (i + incur) % m;
        V const* s = S_(j);
        V const* y = Y_(j);
        R const beta = static_cast<R>(rho[j]) * wdot<MIXED>(y, out, M);
        V const ab = static_cast<V>(static_cast<R>(alpha[j]) - beta);
        for (int e = lane; e < M; e += 32) out[e] += ab * s[e];
      }
      __syncwarp();
      ++k;
    }

    // trans_proj (rotor.cpp:33-47), warp 0: remove the mean per component.
    template <typename T>
    __device__ void trans_proj(Ctx const& c, T* x) {
      double p[3] = {0.0, 0.0, 0.0};
      for (int e = threadIdx.x; e < c.M; e += 32) p[e % 3] += static_cast<double>(x[e]);
      for (double& v : p) v = warp_sum(v);
      double const inv = lane0([&] { return 1.0 / static_cast<double>(c.na); });
      double const q[3] = {p[0] * inv, p[1] * inv, p[2] * inv};
      for (int e = threadIdx.x; e < c.M; e += 32) x[e] = static_cast<T>(static_cast<double>(x[e]) - q[e % 3]);
      __syncwarp();
    }

    // Broadcast of warp 0's decision to the block.
    __device__ inline int block_action(Blk& sh, int act) {
      if (threadIdx.x == 0) sh.action = act;
      __syncthreads();
      int const a = sh.action;
      __syncthreads();
      return a;
    }

    // ------------------------------------------------------------------ Rotor::eff_gradient

    // Returns true on a device-side error; the curvature lands in sh.curv. Vectors are V (binary32 in
    // binary32-pair searches); every scalar is cast to V before it scales a vector, so the per-element
    // work stays in V.
    template <bool MIXED, int LPA>
    __device__ bool eff_gradient(Ctx const& c, TablesView const& tb, SearchOpts const& o, Blk& sh) {
      using V = Vt<MIXED>;
      using R = Red<MIXED>;
      int const M = c.M;
      bool const lead = threadIdx.x < 32;
      int const lane = threadIdx.x & 31;
      V* ax = vp<MIXED>(c.V(V_AX));
      V* g0 = vp<MIXED>(c.V(V_G0));
      V* g1 = vp<MIXED>(c.V(V_G1));
      V* g1p = vp<MIXED>(c.V(V_G1P));
      V* dprev = vp<MIXED>(c.V(V_DPREV));
      V* axp = vp<MIXED>(c.V(V_AXP));
      V* th = vp<MIXED>(c.V(V_TH));
      V* eff = vp<MIXED>(c.V(V_EFF));
      double const dr = o.delta_r;
      V const drv = static_cast<V>(dr);
      int kR = 0;
      double curv = 0;
      if (gradient<MIXED, LPA>(c, tb, sh, g0)) return true;
      if (lead) {
        for (int e = lane; e < M; e += 32) dprev[e] = -drv * ax[e];
        __syncwarp();
        wlist_update(c, dprev, 1.0);
      }
      if (gradient<MIXED, LPA>(c, tb, sh, g1)) return true;
      for (int i = 0;; i++) {
        // rotation plane and trial angle (warp 0)
        double theta_1 = 0, b_1 = 0, c_x0 = 0;
        int act = ACT_GO;
        if (lead) {
          V* dg = g1p;  // scratch until the trial gradient is evaluated
          R tl = 0;
          for (int e = lane; e < M; e += 32) {
            dg[e] = g1[e] - g0[e];
            tl += static_cast<R>(dg[e]) * static_cast<R>(ax[e]);
          }
          V const t = static_cast<V>(wsum<MIXED>(tl));
          for (int e = lane; e < M; e += 32) dg[e] -= t * ax[e];
          __syncwarp();
          if (c.S->count_frozen == 0) trans_proj(c, dg);
          newton<MIXED>(c, c.mR, kR, c.sR(0), c.yR(0), sh.rhoR, sh.alphaR, vp<MIXED>(c.V(V_PXR)),
                        vp<MIXED>(c.V(V_PGR)), static_cast<V const*>(ax), static_cast<V const*>(dg), th);
          V const tp = static_cast<V>(wdot<MIXED>(th, ax, M));
          R nl = 0;
          for (int e = lane; e < M; e += 32) {
            th[e] -= tp * ax[e];
            nl += static_cast<R>(th[e]) * static_cast<R>(th[e]);
          }
          double const nn = wsum<MIXED>(nl);
          V const inv = static_cast<V>(scal<MIXED>([&] { return rsqrtf(static_cast<float>(nn)); },
                                                   [&] { return 1 / sqrt(nn); }));
          R bl = 0, cl = 0;
          for (int e = lane; e < M; e += 32) {
            th[e] *= inv;
            V const df = g1[e] - g0[e];
            bl += static_cast<R>(df) * static_cast<R>(th[e]);
            cl += static_cast<R>(df) * static_cast<R>(ax[e]);
          }
          double const b = wsum<MIXED>(bl), cc = wsum<MIXED>(cl);
          b_1 = scal<MIXED>([&] { return static_cast<float>(b) / static_cast<float>(dr); }, [&] { return b / dr; });
          c_x0 = scal<MIXED>([&] { return static_cast<float>(cc) / static_cast<float>(dr); }, [&] { return cc / dr; });
          double const b1 = b_1, cx0 = c_x0;
          if (MIXED) {  // rotation angles in binary32 (see below)
            theta_1 = -0.5 * static_cast<double>(atanf(static_cast<float>(b1) / fabsf(static_cast<float>(cx0))));
          } else {
            theta_1 = lane0([&] { return -0.5 * atan(b1 / fabs(cx0)); });
          }
          if (fabs(theta_1) < o.theta_tol || (i >= o.iter_max_rot && c_x0 < 0) || i > 10 * o.iter_max_rot) {
            curv = c_x0;
            act = ACT_STOP;
          } else {
            double const t1 = theta_1;
            V c1, s1;
            if (MIXED) {
              float sf, cf;
              sincosf(static_cast<float>(t1), &sf, &cf);
              c1 = static_cast<V>(cf);
              s1 = static_cast<V>(sf);
            } else {
              c1 = static_cast<V>(lane0([&] { return cos(t1); }));
              s1 = static_cast<V>(lane0([&] { return sin(t1); }));
            }
            for (int e = lane; e < M; e += 32) {
              axp[e] = ax[e] * c1 + th[e] * s1;
              V const nd = -drv * axp[e];
              V const upd = nd - dprev[e];
              dprev[e] = nd;
              comp(c.xl[c.aatom[e / 3]], e % 3) -= static_cast<double>(upd);
            }
          }
        }
        if (block_action(sh, act) == ACT_STOP) break;
        if (gradient<MIXED, LPA>(c, tb, sh, g1p)) return true;
        if (lead) {
          R cxl = 0;
          for (int e = lane; e < M; e += 32) cxl += static_cast<R>(g1p[e] - g0[e]) * static_cast<R>(axp[e]);
          double const cx = wsum<MIXED>(cxl);
          double const t1 = theta_1, b1 = b_1, cx0 = c_x0;
          // the rotor's scalar trigonometry (rotor.cpp:120-134)
          double sc[6];
          if (MIXED) {
            // Rotor angles in binary32: the curvatures c_x0, c_x1 and b_1 come from the dots above; the
            // angle arithmetic of rotor.cpp:120-134 is carried in binary32 (errors ~1e-7 rad, far below
            // the rotor's angle tolerance), with 1 - cos(2x) written as 2 sin^2(x) to keep its precision.
            float const c_x1 = static_cast<float>(cx) / static_cast<float>(dr);
            float const f1 = static_cast<float>(t1);
            float s1f, c1f, s2f, c2f;
            sincosf(f1, &s1f, &c1f);
            sincosf(2.f * f1, &s2f, &c2f);
            float const a_1 = (static_cast<float>(cx0) - c_x1 + static_cast<float>(b1) * s2f) / (2.f * s1f * s1f);
            float tm = 0.5f * atanf(static_cast<float>(b1) / a_1);
            float sm2, cm2;
            sincosf(2.f * tm, &sm2, &cm2);
            float const sm1 = sinf(tm);
            if (-2.f * a_1 * sm1 * sm1 + static_cast<float>(b1) * sm2 > 0.f) tm += 1.57079632679489661923f;
            float smf, cmf;
            sincosf(tm, &smf, &cmf);
            sc[0] = cmf;
            sc[1] = smf;
            sc[2] = sinf(f1 - tm) / s1f;
            sc[3] = smf / s1f;
            sc[4] = 1.f - cmf - smf * tanf(0.5f * f1);
            sc[5] = tm;
          } else {
            if (lane == 0) {
              double const c_x1 = cx / dr;
              double const a_1 = (cx0 - c_x1 + b1 * sin(2 * t1)) / (1 - cos(2 * t1));
              double theta_min = 0.5 * atan(b1 / a_1);
              if (a_1 * cos(2 * theta_min) - a_1 + b1 * sin(2 * theta_min) > 0) theta_min += M_PI / 2;
              double const cm = cos(theta_min), sm = sin(theta_min);
              sc[0] = cm;
              sc[1] = sm;
              sc[2] = sin(t1 - theta_min) / sin(t1);
              sc[3] = sm / sin(t1);
              sc[4] = 1 - cm - sm * tan(0.5 * t1);
              sc[5] = theta_min;
            }
#pragma unroll
            for (int q = 0; q < 6; ++q) sc[q] = __shfl_sync(FULL, lane == 0 ? sc[q] : 0.0, 0);
          }
          V const cm = static_cast<V>(sc[0]), sm = static_cast<V>(sc[1]), w1 = static_cast<V>(sc[2]),
                  w1p = static_cast<V>(sc[3]), w0 = static_cast<V>(sc[4]);
          double const theta_min = sc[5];
          R ql = 0;
          for (int e = lane; e < M; e += 32) {
            ax[e] = ax[e] * cm + th[e] * sm;
            g1[e] = w1 * g1[e] + w1p * g1p[e] + w0 * g0[e];
            ql += static_cast<R>(g1[e] - g0[e]) * static_cast<R>(ax[e]);
          }
          __syncwarp();
          if (fabs(theta_min) < o.theta_tol) {
            double const q = wsum<MIXED>(ql);
            curv = scal<MIXED>([&] { return static_cast<float>(q) / static_cast<float>(dr); }, [&] { return q / dr; });
            act = ACT_STOP;
          }
        }
        if (block_action(sh, act) == ACT_STOP) break;
      }
      if (lead) {
        wlist_update(c, dprev, -1.0);  // xl -= -dprev: back to the centre
        V const p = static_cast<V>(wdot<MIXED>(g0, ax, M));
        bool const parallel_only = !o.relax_in_convex && curv > 0;
        for (int e = lane; e < M; e += 32) eff[e] = parallel_only ? -p * ax[e] : g0[e] - V(2) * p * ax[e];
        __syncwarp();
        if (c.S->count_frozen == 0) trans_proj(c, eff);
        if (lane == 0) sh.curv = curv;
      }
      __syncthreads();
      return false;
    }

    // ------------------------------------------------------------------ one search

    // Binary32-pair searches keep the axis in binary32 (Vt) while they run; the host writes and reads it
    // in binary64. Converts the V_AX slot in place (to_v: binary64 -> V, else V -> binary64) through the
    // V_G0 slot, which holds no state at the start or the end of a search. All threads.
    template <bool MIXED>
    __device__ void axis_storage(Ctx const& c, bool to_v) {
      double* axd = c.V(V_AX);
      double* tmp = c.V(V_G0);
      Vt<MIXED>* axv = vp<MIXED>(axd);
      __syncthreads();
      for (int e = threadIdx.x; e < c.M; e += blockDim.x) tmp[e] = to_v ? axd[e] : static_cast<double>(axv[e]);
      __syncthreads();
      for (int e = threadIdx.x; e < c.M; e += blockDim.x) {
        if (to_v) {
          axv[e] = static_cast<Vt<MIXED>>(tmp[e]);
        } else {
          axd[e] = tmp[e];
        }
      }
      __syncthreads();
    }

    template <bool MIXED, int LPA>
    __device__ void run(BatchView const& bv, Blk& sh, Ctx& cs, int sidx) {
      SearchDev* S = bv.S + sidx;
      if (S->stage == STAGE_DONE) return;
      SearchOpts const& o = bv.o;
      Ctx cl;  // this thread's copy while it is set up; the block then reads the shared one (cs)
      cl.S = S;
      cl.n = S->n;
      cl.na = S->na;
      cl.M = 3 * S->na;
      bool const dimer = S->mode == MODE_DIMER;
      cl.mT = dimer ? o.mT : o.mL;
      cl.mR = dimer ? o.mR : 0;
      cl.xl = S->xl;
      cl.pk = S->pk;
      cl.ty = S->type;
      cl.aatom = S->aatom;
      cl.ncnt = S->ncnt;
      cl.nbr = S->nbr;
      cl.v = S->vec;
      cl.hist = S->hist;
      cl.mob = S->mob;
      cl.rho0 = S->rho0;
      cl.need = S->need;
      cl.mark = S->mark;
      cl.dacc = S->dacc;
      cl.rc2 = o.r_cut * o.r_cut;
      cl.rc2f = static_cast<float>(cl.rc2);
      cl.periodic = S->periodic_any != 0;
      for (int k = 0; k < 3; ++k) {
        cl.L[k] = S->L[k];
        cl.invL[k] = 1.0 / S->L[k];
        cl.Lf[k] = static_cast<float>(S->L[k]);
        cl.per[k] = S->per[k] != 0;
        cl.shift[k] = S->shift[k];
      }
      // Stage the search's vectors, positions and binary32 slot records in this CTA's dynamic shared
      // memory for the launch, as far as they fit (in that order). All three are rewritten every step,
      // so from global memory each dependent step would be an L2 round trip.
      extern __shared__ __align__(128) unsigned char dsm[];
      std::size_t const vb = static_cast<std::size_t>(N_VEC + 2 * cl.mT + 2 * cl.mR) * static_cast<std::size_t>(cl.M);
      std::size_t const vbr = (vb * sizeof(double) + 127) / 128 * 128;
      std::size_t const xb = static_cast<std::size_t>(cl.n) * sizeof(D4);
      std::size_t const pb = static_cast<std::size_t>(cl.n) * sizeof(Packed);
      std::size_t const cap = static_cast<std::size_t>(bv.smem_bytes);
      bool const st_v = vbr <= cap, st_x = vbr + xb <= cap, st_p = vbr + xb + pb <= cap;
      if (st_v) {
        double* v = reinterpret_cast<double*>(dsm);
        for (std::size_t e = threadIdx.x; e < vb; e += blockDim.x) v[e] = S->vec[e];
        cl.v = v;
      }
      if (st_x) {
        double2* x = reinterpret_cast<double2*>(dsm + vbr);
        double2 const* g = reinterpret_cast<double2 const*>(S->xl);
        for (std::size_t e = threadIdx.x; e < xb / 16; e += blockDim.x) x[e] = g[e];
        cl.xl = reinterpret_cast<D4*>(x);
      }
      if (st_p) {
        float4* q = reinterpret_cast<float4*>(dsm + vbr + xb);
        float4 const* g = reinterpret_cast<float4 const*>(S->pk);
        for (std::size_t e = threadIdx.x; e < pb / 16; e += blockDim.x) q[e] = g[e];
        cl.pk = reinterpret_cast<Packed*>(q);
      }
      for (int h = threadIdx.x; h < MAX_HIST; h += blockDim.x) {
        sh.rhoT[h] = S->rhoT[h];
        sh.alphaT[h] = S->alphaT[h];
      }
      if (threadIdx.x == 0) cs = cl;
      __syncthreads();
      Ctx const& c = cs;
      TablesView const& tb = bv.tb;
      double const skin = S->rc_list - (dimer ? o.r_cut + 2 * o.delta_r : o.r_cut);
      using V = Vt<MIXED>;
      double* X = c.V(V_X);
      V* eff = vp<MIXED>(c.V(V_EFF));
      V* hg = vp<MIXED>(c.V(V_HG));
      int const M = c.M;
      bool const lead = threadIdx.x < 32;
      int const lane = threadIdx.x & 31;
      if (threadIdx.x == 0) {
        sh.flag = 0;
        sh.n_need = S->n_need;
      }
      __syncthreads();

      // warp 0 holds the search's scalars
      int kT = S->kT, it = S->it;
      double trust = S->trust, acc = S->acc, convex = S->convex, curv = S->curv;
      int exit_code = FLYGPU_EXIT_UNINIT;
      bool done = false, err = false;

      if (S->stage == STAGE_INIT) {
        for (int i = threadIdx.x; i < c.n; i += blockDim.x) {
          D4& p = c.xl[i];
          p.x = p.x - c.L[0] * floor(p.x * c.invL[0]);
          p.y = p.y - c.L[1] * floor(p.y * c.invL[1]);
          p.z = p.z - c.L[2] * floor(p.z * c.invL[2]);
          pack_one(c, i);
          c.dacc[i] = 0;
        }
        if (MIXED && dimer) axis_storage<true>(c, true);  // the host wrote the axis in binary64
        err = rebuild(c, sh, S->rc_list);
        static_density<MIXED>(c, tb, sh);
        __syncthreads();
        err = err || sh.flag != 0;
        kT = 0;
        it = 0;
        acc = 0;
        convex = 0;
        curv = 0;
        if (!err) {
          if (dimer) {
            err = eff_gradient<MIXED, LPA>(c, tb, o, sh);
            curv = sh.curv;
            trust = o.min_trust;
          } else {
            err = gradient<MIXED, LPA>(c, tb, sh, eff);
            trust = o.min_trust_l;
          }
        }
      }

      int const max_steps = dimer ? o.max_steps : o.iter_max_l;
      double const f2 = dimer ? o.f2norm : o.f2norm_l;
      int steps_here = 0;
      while (!err) {
        int act = ACT_GO;
        if (lead) {
          if (it >= max_steps) {
            exit_code = dimer ? FLYGPU_EXIT_ITER_MAX : 1;
            done = true;
            act = ACT_STOP;
          } else if (bv.budget > 0 && steps_here >= bv.budget) {
            act = ACT_STOP;
          } else {
            double const mag = wdot<MIXED>(eff, eff, M);
            if (mag < f2 * f2) {
              exit_code = dimer ? FLYGPU_EXIT_SUCCESS : 0;
              done = true;
              act = ACT_STOP;
            } else if (dimer && convex >= o.convex_max) {
              exit_code = FLYGPU_EXIT_CONVEX;
              done = true;
              act = ACT_STOP;
            } else if (dimer && o.use_history && S->n_hist > 0 && it % o.hist_check_freq == 0) {
              double ctheta = -1;
              double const* im = c.V(V_INMIN);
              for (int h = 0; h < S->n_hist; ++h) {
                double const* sp = c.hist + static_cast<std::int64_t>(h) * M;
                double q0 = 0, q1 = 0, q2 = 0;
                for (int e = lane; e < M; e += 32) {
                  double const d1 = X[e] - im[e], d2 = sp[e] - im[e];
                  q0 += d1 * d2;
                  q1 += d2 * d2;
                  q2 += d1 * d1;
                }
                // plus the static atoms' constant shares (the reference dots over all 3n coordinates)
                double const* hs = c.hist + static_cast<std::int64_t>(S->n_hist) * M + 2 * h;
                q0 = warp_sum(q0) + hs[0];
                q1 = warp_sum(q1) + hs[1];
                q2 = warp_sum(q2) + S->hist_static_on2;
                double const ct = ctheta;
                ctheta = lane0([&] { return fmax(ct, q0 / (sqrt(q1) * sqrt(q2))); });
                double const cth = ctheta;
                if (lane0([&] { return cth > cos(S->theta_tol_hist) ? 1.0 : 0.0; }) != 0.0) {
                  exit_code = FLYGPU_EXIT_COLLISION;
                  done = true;
                  act = ACT_STOP;
                  break;
                }
              }
            }
          }
          if (act == ACT_GO) {
            newton<MIXED>(c, c.mT, kT, c.sT(0), c.yT(0), sh.rhoT, sh.alphaT, c.V(V_PXT), vp<MIXED>(c.V(V_PGT)),
                          static_cast<double const*>(X), static_cast<V const*>(eff), hg);
            double const nrm = wdot<MIXED>(hg, hg, M);
            double const tr = trust;
            V const sc = static_cast<V>(scal<MIXED>([&] { return fminf(1.f, static_cast<float>(tr) * rsqrtf(static_cast<float>(nrm))); },
                                                    [&] { return fmin(1.0, tr / sqrt(nrm)); }));
            Red<MIXED> hl = 0;
            for (int e = lane; e < M; e += 32) {
              hg[e] *= sc;
              hl += static_cast<Red<MIXED>>(hg[e]) * static_cast<Red<MIXED>>(hg[e]);
              X[e] -= static_cast<double>(hg[e]);
            }
            double const hh = wsum<MIXED>(hl);
            acc += scal<MIXED>([&] { return sqrtf(static_cast<float>(hh)); }, [&] { return sqrt(hh); });
            if (acc > 0.5 * skin) {
              acc = 0;
              act = ACT_REBUILD;
            } else {
              __syncwarp();
              wlist_update(c, hg, 1.0);
            }
          }
        }
        act = block_action(sh, act);
        if (act == ACT_STOP) break;
        if (act == ACT_REBUILD && rebuild_mobile(c, sh, S->rc_list)) {
          err = true;
          break;
        }
        if (dimer) {
          if (eff_gradient<MIXED, LPA>(c, tb, o, sh)) {
            err = true;
            break;
          }
          curv = sh.curv;
        } else if (gradient<MIXED, LPA>(c, tb, sh, eff)) {
          err = true;
          break;
        }
        if (lead) {
          if (dimer) convex = curv > 0 ? convex + 1 : 0;
          double const proj = wdot<MIXED>(eff, hg, M);
          double const ptol = dimer ? o.proj_tol : o.proj_tol_l;
          if (proj < -ptol) {
            trust = fmax(dimer ? o.min_trust : o.min_trust_l, (dimer ? o.shrink_trust : o.shrink_trust_l) * trust);
          } else if (proj > ptol) {
            trust = fmin(dimer ? o.max_trust : o.max_trust_l, (dimer ? o.grow_trust : o.grow_trust_l) * trust);
          }
        }
        ++it;
        ++steps_here;
      }
      // warp 0's verdict for the whole block
      if (threadIdx.x == 0) sh.action = (done ? 1 : 0) | (err ? 2 : 0);
      __syncthreads();
      int const verdict = sh.action;
      __syncthreads();
      done = (verdict & 1) != 0;
      err = (verdict & 2) != 0;
      if (err && threadIdx.x == 0) S->status = (sh.flag & F_NLIST) ? FLYGPU_NLIST_OVERFLOW : FLYGPU_SPLINE_OOB;
      double e_final = 0;
      if (done && !err) {
        // the energy sums every pair, so static atoms' lists must see the mobile atoms' final places
        if (rebuild(c, sh, S->rc_list)) {
          if (threadIdx.x == 0) S->status = FLYGPU_NLIST_OVERFLOW;
        } else {
          e_final = energy<MIXED, LPA>(c, tb, sh);
        }
      }
      __syncthreads();
      if (MIXED && dimer && (done || err)) axis_storage<true>(c, false);  // the host reads it in binary64
      if (st_v) {
        for (std::size_t e = threadIdx.x; e < vb; e += blockDim.x) S->vec[e] = c.v[e];
      }
      if (st_x) {
        double2 const* x = reinterpret_cast<double2 const*>(c.xl);
        double2* g = reinterpret_cast<double2*>(S->xl);
        for (std::size_t e = threadIdx.x; e < xb / 16; e += blockDim.x) g[e] = x[e];
      }
      if (st_p) {
        float4 const* q = reinterpret_cast<float4 const*>(c.pk);
        float4* g = reinterpret_cast<float4*>(S->pk);
        for (std::size_t e = threadIdx.x; e < pb / 16; e += blockDim.x) g[e] = q[e];
      }
      for (int h = threadIdx.x; h < MAX_HIST; h += blockDim.x) {
        S->rhoT[h] = sh.rhoT[h];
        S->alphaT[h] = sh.alphaT[h];
      }
      if (threadIdx.x == 0) {
        S->kT = kT;
        S->n_need = sh.n_need;
        S->it = it;
        S->trust = trust;
        S->acc = acc;
        S->convex = convex;
        S->curv = curv;
        if (done || err) {
          S->stage = STAGE_DONE;
          S->exit_code = exit_code;
          S->energy = e_final;
        } else {
          S->stage = STAGE_LOOP;
        }
      }
      __syncthreads();
    }

    // One CTA pulls search indices from the batch's atomic work counter until the batch is exhausted.
    template <bool MIXED, int LPA>
    __device__ __forceinline__ void search_items(BatchView const& bv) {
      __shared__ Blk sh;
      __shared__ Ctx cs;
      int const n_items = bv.n_items_dev ? *bv.n_items_dev : bv.n_items;
      for (;;) {
        if (threadIdx.x == 0) sh.item = atomicAdd(bv.work, 1);
        __syncthreads();
        int const item = sh.item;
        __syncthreads();
        if (item >= n_items) break;
        run<MIXED, LPA>(bv, sh, cs, bv.order[item]);
      }
    }

    // The compiler's register allocation (binary32 pairs: ~226 registers, two 128-thread CTAs an SM).
    template <bool MIXED, int LPA>
    __global__ void k_search(BatchView bv) {
      search_items<MIXED, LPA>(bv);
    }

    // At most 128 registers a thread (a few dozen bytes of spills): four 128-thread CTAs an SM. The
    // search is latency-bound (dependent binary64 chains, three dependent loads per pair), so more
    // resident searches per SM is the main lever; the autotuner times both variants.
    template <bool MIXED, int LPA>
    __global__ void __maxnreg__(128) k_search_r128(BatchView bv) {
      search_items<MIXED, LPA>(bv);
    }

  }  // namespace

}  // namespace flygpu

// Defines search_kernels<MIXED, LPA>() in the translation unit that expands it (one per variant, so the
// eight variants compile in parallel).
#define FLYGPU_SEARCH_KERNELS(MIXED, LPA)                                  \
  namespace flygpu {                                                       \
    template <>                                                            \
    SearchKernels search_kernels<MIXED, LPA>() {                           \
      return SearchKernels{{&k_search<MIXED, LPA>, &k_search_r128<MIXED, LPA>}}; \
    }                                                                      \
  }
