// search_plain.cpp -- the plain drop-in path: the reference's host-side searches over the GPU potential.
//
// This is what a reference user gets by adding the GPU EAM as a potential::Generic alternative: the
// search loop of Dimer::find_sp (src/saddle/dimer.cpp:28-171), Rotor::eff_gradient
// (src/saddle/rotor.cpp:33-164), StepLBFGS (src/minimise/LBFGS/lbfgs_core.cpp:29-87) and
// LBFGS::minimise (src/minimise/LBFGS/lbfgs.cpp:29-115) stays on the host over 3N-vectors, and every
// List::rebuild / List::update / EAM::gradient goes through flygpu_list_* / flygpu_eam_* with host
// buffers (one search at a time, a host<->device round trip per gradient).

#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
#include <vector>

#include "internal.hpp"

extern "C" int flygpu_list_rebuild(flygpu_list*, const double*, int64_t);

namespace flygpu {

  namespace {

    using Vec = std::vector<double>;

    double dot(Vec const& a, Vec const& b) {
      double s = 0;
      for (std::size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
      return s;
    }

    void ok(int st, char const* what) {
      if (st != FLYGPU_OK) fail(st, std::string(what) + ": " + flygpu_last_error());
    }

    // The GPU potential as the host search sees it.
    struct GpuPot {
      flygpu_eam* eam;
      flygpu_list* nl = nullptr;
      std::uint32_t const* types;
      std::uint8_t const* frozen;
      int precision;
      long long grad_calls = 0;
      bool types_sent = false;
      ~GpuPot() { flygpu_list_destroy(nl); }
      void make_list(double const* ext, int const* per, double rc) {
        flygpu_list_destroy(nl);
        nl = nullptr;
        ok(flygpu_list_create(ext, per, rc, nullptr, &nl), "List");
        types_sent = false;
      }
      void rebuild(Vec const& x) { ok(flygpu_list_rebuild(nl, x.data(), static_cast<int64_t>(x.size() / 3)), "List::rebuild"); }
      void update(Vec const& d) { ok(flygpu_list_update(nl, d.data()), "List::update"); }
      void gradient(Vec& g) {
        g.resize(static_cast<std::size_t>(3 * flygpu_list_size(nl)));
        ok(flygpu_eam_gradient(eam, nl, types_sent ? nullptr : types, types_sent ? nullptr : frozen, precision, g.data()),
           "EAM::gradient");
        types_sent = true;
        ++grad_calls;
      }
      double energy() {
        double e = 0;
        ok(flygpu_eam_energy(eam, nl, nullptr, nullptr, precision, &e), "EAM::energy");
        return e;
      }
    };

    struct Core {  // StepLBFGS
      int m, k = 0;
      std::vector<Vec> s, y;
      std::vector<double> rho, alpha;
      Vec px, pg, out;
      explicit Core(int n) : m(n), s(static_cast<std::size_t>(n)), y(static_cast<std::size_t>(n)),
                             rho(static_cast<std::size_t>(n)), alpha(static_cast<std::size_t>(n)) {}
      Vec& step(Vec const& x, Vec const& g) {
        std::size_t const N = x.size();
        int const prev = k > 0 ? (k - 1) % m : 0;
        if (k > 0) {
          auto& sp = s[static_cast<std::size_t>(prev)];
          auto& yp = y[static_cast<std::size_t>(prev)];
          sp.resize(N);
          yp.resize(N);
          for (std::size_t i = 0; i < N; ++i) {
            sp[i] = x[i] - px[i];
            yp[i] = g[i] - pg[i];
          }
          rho[static_cast<std::size_t>(prev)] = 1.0 / std::abs(dot(sp, yp));
        }
        px = x;
        pg = g;
        out = g;
        int const incur = k <= m ? 0 : k - m, bound = k <= m ? k : m;
        for (int i = bound - 1; i >= 0; --i) {
          auto const j = static_cast<std::size_t>((i + incur) % m);
          alpha[j] = rho[j] * dot(s[j], out);
          for (std::size_t e = 0; e < N; ++e) out[e] -= alpha[j] * y[j][e];
        }
        if (k > 0) {
          auto const p = static_cast<std::size_t>(prev);
          double const sc = 1.0 / rho[p] / dot(y[p], y[p]);
          for (double& e : out) e *= sc;
        }
        for (int i = 0; i <= bound - 1; ++i) {
          auto const j = static_cast<std::size_t>((i + incur) % m);
          double const beta = rho[j] * dot(y[j], out);
          for (std::size_t e = 0; e < N; ++e) out[e] += (alpha[j] - beta) * s[j][e];
        }
        ++k;
        return out;
      }
    };

    void trans_proj(Vec& x) {
      std::size_t const N = x.size() / 3;
      double p[3] = {0, 0, 0};
      for (std::size_t i = 0; i < N; ++i)
        for (int c = 0; c < 3; ++c) p[c] += x[3 * i + static_cast<std::size_t>(c)];
      double const inv = 1.0 / static_cast<double>(N);
      for (double& e : p) e *= inv;
      for (std::size_t i = 0; i < N; ++i)
        for (int c = 0; c < 3; ++c) x[3 * i + static_cast<std::size_t>(c)] -= p[c];
    }

    double eff_gradient(flygpu_dimer_options const& o, GpuPot& pot, Vec& out, Vec& ax, int count_frozen) {
      std::size_t const N = ax.size();
      Core core(o.rot_n);
      Vec g0, g1, g1p, axp(N), dprev(N), d(N), dg(N), diff(N);
      pot.gradient(g0);
      for (std::size_t e = 0; e < N; ++e) dprev[e] = -o.delta_r * ax[e];
      pot.update(dprev);
      pot.gradient(g1);
      double curv = 0;
      for (int i = 0;; i++) {
        for (std::size_t e = 0; e < N; ++e) dg[e] = g1[e] - g0[e];
        double const t = dot(dg, ax);
        for (std::size_t e = 0; e < N; ++e) dg[e] -= t * ax[e];
        if (count_frozen == 0) trans_proj(dg);
        Vec& th = core.step(ax, dg);
        double const tp = dot(th, ax);
        for (std::size_t e = 0; e < N; ++e) th[e] -= tp * ax[e];
        double const inv = 1 / std::sqrt(dot(th, th));
        for (double& e : th) e *= inv;
        for (std::size_t e = 0; e < N; ++e) diff[e] = g1[e] - g0[e];
        double const b_1 = dot(diff, th) / o.delta_r;
        double const c_x0 = dot(diff, ax) / o.delta_r;
        double const theta_1 = -0.5 * std::atan(b_1 / std::abs(c_x0));
        if (std::abs(theta_1) < o.theta_tol || (i >= o.iter_max_rot && c_x0 < 0) || i > 10 * o.iter_max_rot) {
          curv = c_x0;
          break;
        }
        double const c1 = std::cos(theta_1), s1 = std::sin(theta_1);
        for (std::size_t e = 0; e < N; ++e) {
          axp[e] = ax[e] * c1 + th[e] * s1;
          double const nd = -o.delta_r * axp[e];
          d[e] = nd - dprev[e];
          dprev[e] = nd;
        }
        pot.update(d);
        pot.gradient(g1p);
        for (std::size_t e = 0; e < N; ++e) diff[e] = g1p[e] - g0[e];
        double const c_x1 = dot(diff, axp) / o.delta_r;
        double const a_1 = (c_x0 - c_x1 + b_1 * std::sin(2 * theta_1)) / (1 - std::cos(2 * theta_1));
        double theta_min = 0.5 * std::atan(b_1 / a_1);
        if (a_1 * std::cos(2 * theta_min) - a_1 + b_1 * std::sin(2 * theta_min) > 0) theta_min += M_PI / 2;
        double const cm = std::cos(theta_min), sm = std::sin(theta_min);
        double const w1 = std::sin(theta_1 - theta_min) / std::sin(theta_1), w1p = sm / std::sin(theta_1);
        double const w0 = 1 - cm - sm * std::tan(0.5 * theta_1);
        for (std::size_t e = 0; e < N; ++e) {
          ax[e] = ax[e] * cm + th[e] * sm;
          g1[e] = w1 * g1[e] + w1p * g1p[e] + w0 * g0[e];
        }
        if (std::abs(theta_min) < o.theta_tol) {
          for (std::size_t e = 0; e < N; ++e) diff[e] = g1[e] - g0[e];
          curv = dot(diff, ax) / o.delta_r;
          break;
        }
      }
      for (std::size_t e = 0; e < N; ++e) d[e] = -dprev[e];
      pot.update(d);
      out.resize(N);
      double const p = dot(g0, ax);
      for (std::size_t e = 0; e < N; ++e) out[e] = (!o.relax_in_convex && curv > 0) ? -p * ax[e] : g0[e] - 2 * p * ax[e];
      if (count_frozen == 0) trans_proj(out);
      return curv;
    }

    double skin_of(double frac, double rc) { return std::max(std::pow(frac, 1. / 3.) - 1, 0.0) * rc; }

  }  // namespace

  void search_plain(flygpu_eam* eam, flygpu_dimer_options const& o, flygpu_lbfgs_options const& lo, int precision,
                    flygpu_search_desc const& d, double* pos_out, double* axis_out, flygpu_search_result& r) {
    if (d.n <= 0 || !d.pos || !d.types || !d.frozen) fail(FLYGPU_INVALID_ARG, "bad search description");
    bool const dimer = d.mode == FLYGPU_SEARCH_DIMER;
    if (dimer && !d.axis) fail(FLYGPU_INVALID_ARG, "dimer search without an axis");
    std::size_t const N = static_cast<std::size_t>(3 * d.n);
    GpuPot pot{eam, nullptr, d.types, d.frozen, precision};
    Vec x(d.pos, d.pos + N), eff, g;
    int count_frozen = 0;
    for (int64_t i = 0; i < d.n; ++i) count_frozen += d.frozen[i] != 0;
    r = flygpu_search_result{};
    r.status = FLYGPU_OK;
    if (dimer) {
      Vec ax(d.axis, d.axis + N), in_min(d.in_min ? d.in_min : d.pos, (d.in_min ? d.in_min : d.pos) + N), d1(N), d2(N);
      double const rr = eam->r_cut + o.delta_r * 2;
      double const skin = skin_of(o.skin_frac, rr);
      pot.make_list(d.extents, d.periodic, rr + skin);
      Core core(o.n);
      pot.rebuild(x);
      double curv = eff_gradient(o, pot, eff, ax, count_frozen);
      double trust = o.min_trust, acc = 0, convex = 0;
      int exit_code = FLYGPU_EXIT_ITER_MAX, i = 0;
      for (; i < o.max_steps; ++i) {
        if (dot(eff, eff) < o.f2norm * o.f2norm) {
          exit_code = FLYGPU_EXIT_SUCCESS;
          break;
        }
        if (convex >= o.convex_max) {
          exit_code = FLYGPU_EXIT_CONVEX;
          break;
        }
        if (o.use_history && d.n_hist > 0 && i % o.hist_check_freq == 0) {
          double ctheta = -1;
          bool hit = false;
          for (int h = 0; h < d.n_hist && !hit; ++h) {
            double const* sp = d.hist + static_cast<std::size_t>(h) * N;
            for (std::size_t e = 0; e < N; ++e) {
              d1[e] = x[e] - in_min[e];
              d2[e] = sp[e] - in_min[e];
            }
            ctheta = std::max(ctheta, dot(d1, d2) / (std::sqrt(dot(d2, d2)) * std::sqrt(dot(d1, d1))));
            hit = ctheta > std::cos(d.theta_tol);
          }
          if (hit) {
            exit_code = FLYGPU_EXIT_COLLISION;
            break;
          }
        }
        Vec& hg = core.step(x, eff);
        double const sc = std::min(1.0, trust / std::sqrt(dot(hg, hg)));
        for (double& e : hg) e *= sc;
        acc += std::sqrt(dot(hg, hg));
        for (std::size_t e = 0; e < N; ++e) x[e] -= hg[e];
        if (acc > 0.5 * skin) {
          pot.rebuild(x);
          acc = 0;
        } else {
          pot.update(hg);
        }
        curv = eff_gradient(o, pot, eff, ax, count_frozen);
        convex = curv > 0 ? convex + 1 : 0;
        double const proj = dot(eff, hg);
        if (proj < -o.proj_tol) {
          trust = std::max(o.min_trust, o.shrink_trust * trust);
        } else if (proj > o.proj_tol) {
          trust = std::min(o.max_trust, o.grow_trust * trust);
        }
      }
      r.exit_code = exit_code;
      r.steps = i;
      r.curvature = curv;
      if (axis_out) std::copy(ax.begin(), ax.end(), axis_out);
    } else {
      double const skin = skin_of(lo.skin_frac, eam->r_cut);
      pot.make_list(d.extents, d.periodic, eam->r_cut + skin);
      Core core(lo.n);
      pot.rebuild(x);
      pot.gradient(g);
      double trust = lo.min_trust, acc = 0;
      int i = 0;
      r.exit_code = 1;
      for (; i < lo.iter_max; ++i) {
        if (dot(g, g) < lo.f2norm * lo.f2norm) {
          r.exit_code = 0;
          break;
        }
        Vec& hg = core.step(x, g);
        double const sc = std::min(1.0, trust / std::sqrt(dot(hg, hg)));
        for (double& e : hg) e *= sc;
        acc += std::sqrt(dot(hg, hg));
        for (std::size_t e = 0; e < N; ++e) x[e] -= hg[e];
        if (acc > 0.5 * skin) {
          pot.rebuild(x);
          acc = 0;
        } else {
          pot.update(hg);
        }
        pot.gradient(g);
        double const proj = dot(g, hg);
        if (proj < -lo.proj_tol) {
          trust = std::max(lo.min_trust, lo.shrink_trust * trust);
        } else if (proj > lo.proj_tol) {
          trust = std::min(lo.max_trust, lo.grow_trust * trust);
        }
      }
      r.steps = i;
      if (axis_out) std::fill(axis_out, axis_out + N, 0.0);
    }
    pot.rebuild(x);
    r.energy = pot.energy();
    r.grad_calls = pot.grad_calls;
    if (pos_out) std::copy(x.begin(), x.end(), pos_out);
  }

}  // namespace flygpu

extern "C" int flygpu_search_plain(flygpu_eam* eam, const flygpu_dimer_options* dimer, const flygpu_lbfgs_options* lbfgs,
                                   int precision, const flygpu_search_desc* desc, double* pos_out, double* axis_out,
                                   flygpu_search_result* result) {
  try {
    if (!eam || !desc || !result) flygpu::fail(FLYGPU_INVALID_ARG, "null argument");
    flygpu_dimer_options d;
    flygpu_lbfgs_options l;
    flygpu_dimer_options_default(&d);
    flygpu_lbfgs_options_default(&l);
    if (dimer) d = *dimer;
    if (lbfgs) l = *lbfgs;
    flygpu::search_plain(eam, d, l, precision, *desc, pos_out, axis_out, *result);
    return FLYGPU_OK;
  } catch (flygpu::Error const& e) {
    flygpu::set_error(e.msg);
    return e.status;
  } catch (std::exception const& e) {
    flygpu::set_error(e.what());
    return FLYGPU_INVALID_ARG;
  }
}
