// hessian.cu -- EAM Hessian, mass weighting and eigenvalues (compiled with -fmad=false).
//
// Restates EAM::hessian (src/potential/EAM/eam.cpp:122-233) on the device. Pass 1, one warp per atom b
// (active and frozen): rho_b = sum_a phi(t_a, t_b)(r) and mu_b = -sum_a phi'(t_a, t_b)(r) dr / r
// (A.13), with F'(rho_b) and F''(rho_b); it also keeps every pair's distance, phi' and destination key
// for pass 2. Pass 2, one CTA per active atom z, writes only column block z of the dense 3n x 3n matrix
// (row-major; the rows of atom a are 3a..3a+2):
//   H(z,z) = F''_z mu_z mu_z^T + sum_a [A 1 - ABFpp dr dr^T]                           (A.15, A.14)
//   H(a,z) += -BArr dr dr^T - A 1 + ur dr mu_z^T - ru mu_a dr^T       for active a > z
//   H(g,z) -= F''_a phi'(t_z,t_a)(r) phi'(t_g,t_a)(r_ag) / (r r_ag) dr_ag dr^T
//             for every neighbour g of a that is active with g > z, or a periodic image of z itself.
// Neighbours come from the list in the reference's visiting order and every coefficient is formed in
// the reference's operation order. The serial loop's contributions (for each a: the (z,z) term, the
// (a,z) term, then the (g,z) terms) are queued in that order; each destination block's contributions
// are applied in queue order (by occurrence levels, the (z,z) block as its own chain). So every
// element receives the reference's contributions in the reference's order, and the result is the
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

    // Pass 1: rho, mu, F'(rho) and F''(rho) of every atom, one warp (CTA) per atom b. Each lane forms the
    // terms of one neighbour (a long dependent chain of binary64 operations: square root, table lookup,
    // three divisions); lane 0 then adds the 32 terms in list order, the reference's operations and order
    // (eam.cpp:131-149). The pair's distance and phi'(t_a, t_b)(r) are kept for pass 2, which needs them
    // for every pair (a, g) once per column z; pr < 0 marks a pair outside the spline's range.
    __global__ void __launch_bounds__(32)
        k_hess_rho(TablesView tb, std::int64_t n, long long const* __restrict__ offs, int const* __restrict__ idx,
                   double const* __restrict__ dr, std::uint32_t const* __restrict__ types,
                   std::uint8_t const* __restrict__ frozen, double* __restrict__ rho_mu, double* __restrict__ fder,
                   double* __restrict__ pr, double* __restrict__ pfp, int* __restrict__ key, int* __restrict__ err) {
      __shared__ double sv[4][32];
      std::int64_t const b = blockIdx.x;
      int const lane = threadIdx.x;
      if (b >= n) return;
      std::uint32_t const t_b = types[b];
      double rho = 0, m0 = 0, m1 = 0, m2 = 0;
      bool bad = false;
      long long const k0 = offs[b], k1 = offs[b + 1];
      for (long long base = k0; base < k1; base += 32) {
        long long const k = base + lane;
        bool const live = k < k1;
        bool ok = false;
        if (live) {
          double const x = dr[3 * k], y = dr[3 * k + 1], z = dr[3 * k + 2];
          double const r = sqrt((x * x + y * y) + z * z);
          Lookup l;
          ok = fetch(r, tb.inv_dR, tb.dR, tb.nR, l);
          int const a = idx[k];
          key[k] = ok && !frozen[a] ? a : -1;
          if (ok) {
            D4 const* ph = phi_t(tb, types[a], t_b);
            double const fp = fp_of(ph, l);
            sv[0][lane] = f_of(ph, l);
            sv[1][lane] = fp * x / r;
            sv[2][lane] = fp * y / r;
            sv[3][lane] = fp * z / r;
            pr[k] = r;
            pfp[k] = fp;
          } else {
            pr[k] = -1;
            pfp[k] = 0;
          }
        }
        unsigned const okm = __ballot_sync(0xffffffffu, ok);
        int const cnt = k1 - base < 32 ? static_cast<int>(k1 - base) : 32;
        __syncwarp();
        if (lane == 0)
          for (int j = 0; j < cnt; ++j) {
            if (!((okm >> j) & 1u)) {
              bad = true;
              continue;
            }
            rho += sv[0][j];
            m0 -= sv[1][j];
            m1 -= sv[2][j];
            m2 -= sv[3][j];
          }
        __syncwarp();
      }
      if (lane != 0) return;
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

    // Pass 2 shape: threads per column CTA, flat slots each thread enumerates per window, the items a
    // window can queue, the neighbours a of z whose coefficients one chunk holds, and the slots of the
    // window's destination table.
    constexpr int COL_T = 256;
    constexpr int COL_SLOTS = 4;
    constexpr int COL_WORK = COL_T - 32;  // threads of warps 1.. (values) and 0.. (levels): all but one warp
    constexpr int COL_W = COL_T * COL_SLOTS;
    constexpr int COL_KC = COL_T;
    constexpr int COL_HASH = 2 * COL_W;

    struct ColShared {
      // neighbour j of the chunk (a_j = idx[k], k = chunk start + j)
      double d[COL_KC][3];
      double r[COL_KC], ddFg[COL_KC];
      double zz[COL_KC][9], az[COL_KC][9];  // the (z,z) and (a_j,z) terms, added as they stand
      long long goff[COL_KC];
      int a[COL_KC];
      int pre[COL_KC + 1];  // first flat slot of neighbour j: slot 0 (z,z), slot 1 (a_j,z), then a_j's neighbours
      int wsum[COL_T / 32];
      unsigned char az_use[COL_KC];
      // the window's queue of items, in the reference's order
      double v[COL_W][9];
      long long q[COL_W];
      int dest[COL_W];
      short j[COL_W];
      short occ[COL_W];  // how often the item's destination block occurs earlier in the window
      short lst[COL_W];  // the items other than (z,z) ones, by occurrence
      short zl[COL_W];   // the items of block (z,z), in order
      signed char kind[COL_W];  // 0: (z,z) add, 1: (a,z) add, 2: (g,z) subtract
      // occurrences so far of each destination block in the window (open addressing on the atom index)
      int hkey[COL_HASH];
      short hcnt[COL_HASH];
      int lvo[COL_W + 1];  // first entry of each occurrence level in lst
      int lvc[COL_W];      // items per level, then the scatter cursors
      int nz, maxocc;
    };

    // Exclusive prefix sum of v over the CTA (COL_T threads), and the total.
    __device__ inline int col_scan(int v, int* wsum, int& total) {
      int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
      int x = v;
      for (int o = 1; o < 32; o <<= 1) {
        int const y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      __syncthreads();  // earlier readers of wsum are done
      if (lane == 31) wsum[warp] = x;
      __syncthreads();
      int off = 0, tot = 0;
      for (int w = 0; w < COL_T / 32; ++w) {
        int const sw = wsum[w];
        if (w < warp) off += sw;
        tot += sw;
      }
      total = tot;
      return off + x - v;
    }

    // Barrier of every warp but the last (COL_WORK threads); the last warp meanwhile runs the (z,z) chain.
    __device__ inline void bar_levels() { asm volatile("bar.sync 1, %0;" ::"n"(COL_WORK) : "memory"); }

    // Pass 2: column block z, one CTA per active atom (cols lists them). The reference's serial loop over
    // z's neighbours a adds, for each a in list order, the (z,z) term, the (a,z) term, then one (g,z) term
    // per neighbour g of a that qualifies. Here the CTA forms every a's coefficients at once, enumerates
    // that sequence of items as flat slots, compacts the items that apply into a queue (order kept), and
    // forms their values densely. Each queued item then gets its occurrence number: how often its
    // destination block occurs earlier in the window. Items of one occurrence level have distinct
    // destinations, so every warp but the last applies level after level, every (item, element) update of
    // a level in parallel; the last warp meanwhile adds the (z,z) block's items one after another in queue
    // order. So every element receives the reference's contributions in the reference's order. The
    // column block accumulates in shared memory (in_smem, rows of 3 doubles) or in place in H.
    __global__ void __launch_bounds__(COL_T)
        k_hess_col(TablesView tb, std::int64_t n, int const* __restrict__ cols, long long const* __restrict__ offs,
                   int const* __restrict__ idx, double const* __restrict__ dr, std::uint32_t const* __restrict__ types,
                   std::uint8_t const* __restrict__ frozen, double const* __restrict__ rho_mu,
                   double const* __restrict__ fder, double const* __restrict__ pr, double const* __restrict__ pfp,
                   int const* __restrict__ key, double* __restrict__ H, int in_smem, int* __restrict__ err) {
      extern __shared__ __align__(16) unsigned char col_smem[];
      ColShared& S = *reinterpret_cast<ColShared*>(col_smem);
      double* const scol = reinterpret_cast<double*>(col_smem + sizeof(ColShared));
      int const t = threadIdx.x, lane = t & 31, warp = t >> 5;
      unsigned const lt = (1u << lane) - 1u;
      std::int64_t const z = cols[blockIdx.x];
      if (z >= n || frozen[z]) return;  // the same for the whole CTA
      std::int64_t const N = 3 * n;
      double* const colp = in_smem ? scol : H + 3 * z;  // element (row, c) of the column block
      std::int64_t const cs = in_smem ? 3 : N;
      if (in_smem)
        for (std::int64_t e = t; e < 9 * n; e += COL_T) scol[e] = 0;
      for (int h = t; h < COL_HASH; h += COL_T) S.hkey[h] = -1;
      for (int h = t; h < COL_W; h += COL_T) S.lvc[h] = 0;
      std::uint32_t const tz = types[z];
      double const mz[3] = {rho_mu[4 * z + 1], rho_mu[4 * z + 2], rho_mu[4 * z + 3]};
      double const fz_p = fder[2 * z], fz_pp = fder[2 * z + 1];
      bool bad = false;
      __syncthreads();
      if (t < 9) colp[(3 * z + t / 3) * cs + t % 3] = (fz_pp * mz[t / 3]) * mz[t % 3];
      long long const kz0 = offs[z], kz1 = offs[z + 1];
      for (long long kb = kz0; kb < kz1; kb += COL_KC) {
        int const nk = kz1 - kb < COL_KC ? static_cast<int>(kz1 - kb) : COL_KC;
        int size = 0;
        if (t < nk) {
          long long const k = kb + t;
          int const a = idx[k];
          double const d[3] = {dr[3 * k], dr[3 * k + 1], dr[3 * k + 2]};
          double const r = pr[k];  // the distance of pair (z, a) as pass 1 formed it; -1 out of range
          Lookup l;
          if (fetch(r, tb.inv_dR, tb.dR, tb.nR, l)) {
            std::uint32_t const ta = types[a];
            double const fa_p = fder[2 * a], fa_pp = fder[2 * a + 1];
            D4 const* p_az = phi_t(tb, ta, tz);
            D4 const* p_za = phi_t(tb, tz, ta);
            D4 const* v_az = v_t(tb, ta, tz);
            double const pza = fp_of(p_za, l);
            double const paz = pfp[k];  // phi'(t_a, t_z)(r), from pass 1
            double const A = (fp_of(v_az, l) + fz_p * paz + fa_p * pza) / r;
            double const B = fpp_of(v_az, l) + fz_p * fpp_of(p_az, l) + fa_p * fpp_of(p_za, l);
            double const ABFpp = (A - B - fa_pp * (pza * pza)) / (r * r);
            for (int i = 0; i < 3; ++i)
              for (int c = 0; c < 3; ++c) S.zz[t][3 * i + c] = (i == c ? A : A * 0.0) - (ABFpp * d[i]) * d[c];
            bool const azu = a > z && !frozen[a];
            if (azu) {
              double const BArr = (B - A) / (r * r);
              double const ur = fz_pp * paz / r;
              double const ru = fa_pp * pza / r;
              double const ma[3] = {rho_mu[4 * a + 1], rho_mu[4 * a + 2], rho_mu[4 * a + 3]};
              for (int i = 0; i < 3; ++i)
                for (int c = 0; c < 3; ++c)
                  S.az[t][3 * i + c] = (((-BArr * d[i]) * d[c] - (i == c ? A : A * 0.0)) + (ur * d[i]) * mz[c]) -
                                       (ru * ma[i]) * d[c];
            }
            for (int c = 0; c < 3; ++c) S.d[t][c] = d[c];
            S.r[t] = r;
            S.ddFg[t] = fa_pp * pza;
            S.goff[t] = offs[a];
            S.a[t] = a;
            S.az_use[t] = azu;
            size = 2 + static_cast<int>(offs[a + 1] - offs[a]);
          } else {
            bad = true;
          }
        }
        int F;
        int const ex = col_scan(size, S.wsum, F);
        if (t < nk) S.pre[t] = ex;
        if (t == 0) S.pre[nk] = F;
        __syncthreads();
        for (int fw = 0; fw < F; fw += COL_W) {
          // enumerate flat slots f0 .. f0 + COL_SLOTS - 1: locate them first, then issue every key load
          // before any is used
          int const f0 = fw + t * COL_SLOTS;
          int oo[COL_SLOTS], jj[COL_SLOTS], gk[COL_SLOTS];
          long long qq[COL_SLOTS];
          int j = 0;
          if (f0 < F) {
            int lo = 0, hi = nk;  // the last j with pre[j] <= f0 (pre[nk] = F > f0)
            while (hi - lo > 1) {
              int const mid = (lo + hi) >> 1;
              if (S.pre[mid] <= f0) lo = mid;
              else hi = mid;
            }
            j = lo;
          }
#pragma unroll
          for (int u = 0; u < COL_SLOTS; ++u) {
            int const f = f0 + u;
            oo[u] = -1;
            jj[u] = 0;
            qq[u] = -1;
            if (f < F) {
              while (S.pre[j + 1] <= f) ++j;
              oo[u] = f - S.pre[j];
              jj[u] = j;
              if (oo[u] >= 2) qq[u] = S.goff[j] + (oo[u] - 2);
            }
          }
#pragma unroll
          for (int u = 0; u < COL_SLOTS; ++u) gk[u] = qq[u] >= 0 ? key[qq[u]] : -1;  // -1: g frozen or out of range
          bool use[COL_SLOTS];
          int kd[COL_SLOTS], dst[COL_SLOTS];
          int cnt = 0;
#pragma unroll
          for (int u = 0; u < COL_SLOTS; ++u) {
            int const o = oo[u], jx = jj[u];
            use[u] = false;
            kd[u] = 2;
            dst[u] = gk[u];
            if (o == 0) {
              use[u] = true;
              kd[u] = 0;
              dst[u] = static_cast<int>(z);
            } else if (o == 1) {
              use[u] = S.az_use[jx];
              kd[u] = 1;
              dst[u] = S.a[jx];
            } else if (o >= 2) {
              long long const q = qq[u];
              bool u2 = gk[u] > z;
              if (gk[u] == z) {  // a periodic image of z itself, unless it is z's own position
                double const sx = S.d[jx][0] + dr[3 * q], sy = S.d[jx][1] + dr[3 * q + 1], sz = S.d[jx][2] + dr[3 * q + 2];
                u2 = sqrt((sx * sx + sy * sy) + sz * sz) > 1e-6;
              }
              use[u] = u2;
            }
            cnt += use[u];
          }
          int nq;
          int pos = col_scan(cnt, S.wsum, nq);
#pragma unroll
          for (int u = 0; u < COL_SLOTS; ++u)
            if (use[u]) {
              S.kind[pos] = static_cast<signed char>(kd[u]);
              S.dest[pos] = dst[u];
              S.j[pos] = static_cast<short>(jj[u]);
              S.q[pos] = qq[u];
              ++pos;
            }
          __syncthreads();
          // values of the (g,z) items (every warp but warp 0, two items an iteration), and meanwhile the occurrence
          // numbers (warp 0, in queue order)
          if (warp > 0)
            for (int i0 = t - 32; i0 < nq; i0 += 2 * COL_WORK) {
              int ii[2] = {i0, i0 + COL_WORK};
              bool g2[2];
              long long q2[2];
              int j2[2];
              double rq[2], fq[2], e2[2][3];
#pragma unroll
              for (int h = 0; h < 2; ++h) {
                g2[h] = ii[h] < nq && S.kind[ii[h]] == 2;
                q2[h] = g2[h] ? S.q[ii[h]] : 0;
                j2[h] = g2[h] ? S.j[ii[h]] : 0;
              }
#pragma unroll
              for (int h = 0; h < 2; ++h)
                if (g2[h]) {
                  long long const q = q2[h];
                  rq[h] = pr[q];
                  fq[h] = pfp[q];
                  e2[h][0] = dr[3 * q];
                  e2[h][1] = dr[3 * q + 1];
                  e2[h][2] = dr[3 * q + 2];
                }
#pragma unroll
              for (int h = 0; h < 2; ++h)
                if (g2[h]) {
                  int const jq = j2[h];
                  double const mag = S.ddFg[jq] / (S.r[jq] * rq[h]) * fq[h];
                  for (int x = 0; x < 3; ++x)
                    for (int c = 0; c < 3; ++c) S.v[ii[h]][3 * x + c] = (mag * e2[h][x]) * S.d[jq][c];
                }
            }
          if (warp == 0) {
            int nzc = 0, mo = -1;
            for (int b0 = 0; b0 < nq; b0 += 32) {
              int const i = b0 + lane;
              bool const live = i < nq;
              int const dd = live ? S.dest[i] : -1;
              bool const isz = live && dd == z;
              unsigned const zb = __ballot_sync(0xffffffffu, isz);
              if (isz) S.zl[nzc + __popc(zb & lt)] = static_cast<short>(i);
              nzc += __popc(zb);
              bool const oth = live && !isz;
              unsigned const peers = __match_any_sync(0xffffffffu, oth ? dd : -1 - lane);
              int const first = __ffs(peers) - 1;
              int base = 0;
              if (oth && lane == first) {
                // find or insert dd; at most COL_W keys in COL_HASH slots, so a free slot exists
                unsigned h = (static_cast<unsigned>(dd) * 2654435761u) >> 21;
                for (int it = 0; it < COL_HASH; ++it) {
                  int const prev = atomicCAS(&S.hkey[h], -1, dd);
                  if (prev == -1) {
                    S.hcnt[h] = 0;
                    break;
                  }
                  if (prev == dd) break;
                  h = (h + 1) & (COL_HASH - 1);
                }
                base = S.hcnt[h];
                S.hcnt[h] = static_cast<short>(base + __popc(peers));
              }
              base = __shfl_sync(0xffffffffu, base, first);
              if (oth) {
                int const oc = base + __popc(peers & lt);
                S.occ[i] = static_cast<short>(oc);
                atomicAdd(&S.lvc[oc], 1);
                mo = max(mo, oc);
              }
              __syncwarp();
            }
            for (int o = 16; o > 0; o >>= 1) mo = max(mo, __shfl_xor_sync(0xffffffffu, mo, o));
            if (lane == 0) {
              S.nz = nzc;
              S.maxocc = mo;
            }
            // offsets of the levels in lst; the counts become the scatter cursors
            int carry = 0;
            for (int b0 = 0; b0 <= mo; b0 += 32) {
              int const L = b0 + lane;
              int const c = L <= mo ? S.lvc[L] : 0;
              int x = c;
              for (int o = 1; o < 32; o <<= 1) {
                int const y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
              }
              if (L <= mo) {
                S.lvo[L] = carry + x - c;
                S.lvc[L] = 0;
              }
              carry += __shfl_sync(0xffffffffu, x, 31);
            }
            if (lane == 0) S.lvo[mo + 1] = carry;
          }
          __syncthreads();
          int const maxocc = S.maxocc, nz = S.nz;
          for (int i = t; i < nq; i += COL_T)
            if (S.dest[i] != z) {
              int const L = S.occ[i];
              S.lst[S.lvo[L] + atomicAdd(&S.lvc[L], 1)] = static_cast<short>(i);
            }
          __syncthreads();
          if (warp < COL_T / 32 - 1) {
            for (int L = 0; L <= maxocc; ++L) {
              int const o0 = S.lvo[L], U = 9 * (S.lvo[L + 1] - o0);
              for (int u = t; u < U; u += COL_WORK) {
                int const i = S.lst[o0 + u / 9], e = u % 9;
                double* const x = colp + (3 * static_cast<std::int64_t>(S.dest[i]) + e / 3) * cs + e % 3;
                int const k2 = S.kind[i];
                if (k2 == 2) *x -= S.v[i][e];
                else *x += S.az[S.j[i]][e];  // kind 1: only (z,z) items are of kind 0
              }
              bar_levels();
            }
          } else if (lane < 9) {
            // block (z,z): its (z,z) terms and any periodic self-image terms, in queue order
            double* const x = colp + (3 * z + lane / 3) * cs + lane % 3;
            double acc = *x;
            for (int m = 0; m < nz; ++m) {
              int const i = S.zl[m];
              if (S.kind[i] == 2) acc -= S.v[i][lane];
              else acc += S.zz[S.j[i]][lane];
            }
            *x = acc;
          }
          __syncthreads();
          // clear the window's destination table and level counts
          for (int h = t; h < COL_HASH; h += COL_T) S.hkey[h] = -1;
          for (int L = t; L <= maxocc; L += COL_T) S.lvc[L] = 0;
        }
      }
      if (in_smem) {
        __syncthreads();
        for (std::int64_t row = t; row < N; row += COL_T)
          for (int c = 0; c < 3; ++c) H[row * N + 3 * z + c] = scol[3 * row + c];
      }
      if (__syncthreads_or(bad) && t == 0) atomicOr(err, ERR_SPLINE_OOB);
    }

    // Hessian::mass_weight: element (row, col) *= 1 / sqrt(m_col m_row). The factor depends only on the
    // two atoms' types, so it is formed once per type pair (the same operations) and each element takes
    // one multiplication: T[a * nt + b] for row type a and column type b.
    __global__ void k_mass_table(double const* __restrict__ mt, int nt, double* __restrict__ T) {
      int const e = blockIdx.x * blockDim.x + threadIdx.x;
      if (e >= nt * nt) return;
      int const a = e / nt, b = e - a * nt;
      T[e] = 1 / sqrt(mt[b] * mt[a]);
    }

    __global__ void k_mass_weight(double* __restrict__ H, std::int64_t N, std::uint32_t const* __restrict__ ty,
                                  double const* __restrict__ T, int nt) {
      for (std::int64_t row = blockIdx.y; row < N; row += gridDim.y) {
        double* const h = H + row * N;
        double const* const Tr = T + static_cast<std::int64_t>(ty[row / 3]) * nt;
        for (std::int64_t col = static_cast<std::int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; col < N;
             col += static_cast<std::int64_t>(gridDim.x) * blockDim.x)
          h[col] *= Tr[ty[col / 3]];
      }
    }

  }  // namespace

  // Dense 3n x 3n Hessian into d_H (device, row-major), on the list's stream. Waits for the list export's
  // pair counts; the Hessian kernels run on after the return (host data is copied from pageable memory,
  // which the driver stages before the copy call returns).
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
    std::vector<int> const cnt = list_export_device(L, E->r_cut, P.offs, P.idx, P.dr);
    long long n_pairs_ll = 0;
    for (int const c : cnt) n_pairs_ll += c;
    P.rho_mu.reserve(4 * static_cast<std::size_t>(n));
    P.fder.reserve(2 * static_cast<std::size_t>(n));
    std::size_t const N = 3 * static_cast<std::size_t>(n);
    FLY_CUDA(cudaMemsetAsync(d_H, 0, sizeof(double) * N * N, s));
    TablesView const tb = E->view();
    std::size_t const n_pairs = static_cast<std::size_t>(n_pairs_ll);
    P.pr.reserve(std::max<std::size_t>(n_pairs, 1));
    P.pfp.reserve(std::max<std::size_t>(n_pairs, 1));
    P.key.reserve(std::max<std::size_t>(n_pairs, 1));
    launch(k_hess_rho, static_cast<unsigned>(n), 32, 0, s, tb, n, P.offs.p, P.idx.p, P.dr.p, L->types.p, L->frozen.p,
           P.rho_mu.p, P.fder.p, P.pr.p, P.pfp.p, P.key.p, L->err.p);
    if (!cols.empty()) {
      // the column block (3n rows of 3 doubles) accumulates in shared memory when it fits. The kernel's
      // shared-memory limit is set to the device's opt-in maximum on every call, the same value from every
      // host thread (the batch entry point runs systems on several), so no caller lowers it under another.
      int dev = 0, optin = 0;
      FLY_CUDA(cudaGetDevice(&dev));
      FLY_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
      std::size_t const col_bytes = sizeof(double) * 9 * static_cast<std::size_t>(n);
      int const in_smem = sizeof(ColShared) + col_bytes <= static_cast<std::size_t>(optin) ? 1 : 0;
      std::size_t const smem = sizeof(ColShared) + (in_smem ? col_bytes : 0);
      FLY_CUDA(cudaFuncSetAttribute(k_hess_col, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
      launch(k_hess_col, static_cast<unsigned>(cols.size()), COL_T, smem, s, tb, n, P.cols.p, P.offs.p, P.idx.p,
             P.dr.p, L->types.p, L->frozen.p, P.rho_mu.p, P.fder.p, P.pr.p, P.pfp.p, P.key.p, d_H, in_smem, L->err.p);
    }
  }

  void hessian_mass_weight(flygpu_eam const* E, flygpu_list* L, double const* type_mass, std::uint32_t const* h_types,
                           double* d_H) {
    std::int64_t const n = L->n;
    if (n == 0) return;
    cudaStream_t const s = L->stream;
    int const nt = E->n_types;
    for (std::int64_t i = 0; i < n; ++i)
      if (h_types[i] >= static_cast<std::uint32_t>(nt)) fail(FLYGPU_INVALID_ARG, "type index out of range");
    std::vector<double> mt(static_cast<std::size_t>(nt));
    for (int t = 0; t < nt; ++t) {
      double const m = type_mass ? type_mass[t] : E->mass[t];
      if (!(m > 0)) {
        // only the masses of types present are used (and checked)
        bool used = false;
        for (std::int64_t i = 0; i < n && !used; ++i) used = h_types[i] == static_cast<std::uint32_t>(t);
        if (used) fail(FLYGPU_INVALID_ARG, "masses must be positive");
      }
      mt[static_cast<std::size_t>(t)] = m;
    }
    DevBuf<double>& dm = L->hs.m3;  // the masses, then the nt x nt factors
    dm.reserve(static_cast<std::size_t>(nt) * (nt + 1));
    DevBuf<std::uint32_t>& dt = L->hs.ty;
    dt.reserve(static_cast<std::size_t>(n));
    FLY_CUDA(cudaMemcpyAsync(dm.p, mt.data(), sizeof(double) * mt.size(), cudaMemcpyHostToDevice, s));
    FLY_CUDA(cudaMemcpyAsync(dt.p, h_types, sizeof(std::uint32_t) * static_cast<std::size_t>(n), cudaMemcpyHostToDevice, s));
    std::int64_t const N = 3 * n;
    launch(k_mass_table, static_cast<unsigned>((nt * nt + 127) / 128), 128, 0, s, dm.p, nt, dm.p + nt);
    unsigned const gx = static_cast<unsigned>(std::min<std::int64_t>((N + 255) / 256, 64));
    unsigned const gy = static_cast<unsigned>(std::min<std::int64_t>(N, 65535));
    launch(k_mass_weight, dim3(gx, gy), 256, 0, s, d_H, N, dt.p, dm.p + nt, nt);
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
