// flyoracle.cpp -- CPU oracle for the openFLY saddle-search inner loop.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker: tests/, __graft_entry__.smoke() and the
// cpu_baseline / --impl reference legs of bench.py load it. The product (openfly_gb300/) never links,
// loads or calls it.
//
// It restates, in plain C++20 + OpenMP (no Eigen), the reference's algorithm for this path:
//   utility/spline.hpp:81-154, src/utility/spline.cpp:27-103          (Spline)
//   potential/EAM/data.hpp:86-116, src/potential/EAM/data.cpp:37-153  (DataEAM, eam/fs parser)
//   system/boxes/orthorhombic.hpp:54-139, boxes/hypergrid.hpp:43-99   (box, grid, ghost images)
//   neigh/adjacent.hpp:40-70                                          (AdjacentCells)
//   src/neigh/list.cpp:37-165, neigh/list.hpp:78,139-154              (List)
//   src/potential/EAM/eam.cpp:33-120                                  (EAM energy / gradient)
//   src/potential/EAM/eam.cpp:122-233                                 (EAM::hessian)
//   src/minimise/LBFGS/lbfgs_core.cpp:29-87                           (StepLBFGS)
//   src/minimise/LBFGS/lbfgs.cpp:29-115                               (LBFGS::minimise)
//   src/saddle/rotor.cpp:33-164                                       (trans_proj, Rotor::eff_gradient)
//   src/saddle/dimer.cpp:28-171                                       (Dimer::find_sp)
//   utility/random.hpp:42-162                                         (Xoshiro256**)
//   src/saddle/find.cpp:1147-1214                                     (Master::perturb, with libstdc++'s
//                                                                      std::normal_distribution as the reference uses it)
//   utility/core.hpp:539-542,634-680                                  (near, gdot, gnorm)
//
// Arithmetic conventions (fixed here so the oracle is deterministic on x86-64 and aarch64):
//   * built with -ffp-contract=off: no fused multiply-add anywhere;
//   * the squared length of a 3-vector is (x*x + y*y) + z*z (Eigen's packet-of-two reduction order);
//   * long reductions (gdot/gnorm over 3N, sums over atoms) are sequential in index order.
// The reference's own build may contract to FMA and vectorise reductions; its known-answer tests
// (tests/potential/EAM/eam.cpp:119,125,141,173-183, tests/potential/EAM/data.cpp:42-43) pin this oracle.
//
// Errors: every entry point returns an int status (0 = ok, 1 = invalid argument, 2 = spline out of
// bounds, 3 = ghost capacity exceeded).

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <exception>
#include <fstream>
#include <limits>
#include <memory>
#include <random>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include <omp.h>

namespace orc {

  enum : int { OK = 0, INVALID = 1, SPLINE_OOB = 2, GHOST_OVERFLOW = 3 };

  struct OutOfBounds : std::runtime_error {
    using std::runtime_error::runtime_error;
  };

  struct Invalid : std::runtime_error {
    using std::runtime_error::runtime_error;
  };

  inline double sq3(double x, double y, double z) { return (x * x + y * y) + z * z; }

  // ---------------------------------------------------------------- Spline (spline.cpp:27-103)

  struct Spline {
    std::vector<std::array<double, 4>> sp;  // {a, b, c, d} per interval
    double dx = 0, inv_dx = 0;

    Spline() = default;

    Spline(std::vector<double> y, double dx_) : dx(dx_), inv_dx(1 / dx_) {
      double last = y.back();
      for (int i = 0; i < 5; i++) y.push_back(last);  // soft pad, spline.cpp:29-33
      std::size_t n = y.size() - 1;
      std::vector<double> a(y), b(n), d(n), alpha(n), c(n + 1), l(n + 1), mu(n + 1), z(n + 1);
      for (std::size_t i = 1; i <= n - 1; ++i) alpha[i] = 3 * (a[i + 1] - 2 * a[i] + a[i - 1]) / dx;
      l[0] = 1;
      mu[0] = 0;
      z[0] = 0;
      for (std::size_t i = 1; i <= n - 1; ++i) {
        l[i] = dx * (4 - mu[i - 1]);
        mu[i] = dx / l[i];
        z[i] = (alpha[i] - dx * z[i - 1]) / l[i];
      }
      l[n] = 1;
      z[n] = 0;
      c[n] = 0;
      for (std::size_t i = 1; i <= n; ++i) {
        std::size_t j = n - i;
        c[j] = z[j] - mu[j] * c[j + 1];
        b[j] = (a[j + 1] - a[j]) / dx - dx * (c[j + 1] + 2 * c[j]) / 3;
        d[j] = (c[j + 1] - c[j]) / (3 * dx);
      }
      sp.reserve(n);
      for (std::size_t i = 0; i < n; ++i) sp.push_back({a[i], b[i], c[i], d[i]});
    }

    // spline.hpp:135-154. A negative argument is reported as out of bounds (the reference casts it
    // to size_t, which is undefined behaviour).
    std::size_t fetch(double x, double& x0) const {
      if (!(x >= 0)) throw OutOfBounds("negative spline argument");
      auto i = static_cast<std::size_t>(x * inv_dx);
      if (i >= sp.size()) throw OutOfBounds("spline argument beyond table");
      x0 = x - static_cast<double>(i) * dx;
      return i;
    }
    double f(double x) const {
      double x0;
      auto const& s = sp[fetch(x, x0)];
      return s[0] + x0 * (s[1] + x0 * (s[2] + x0 * s[3]));
    }
    double fp(double x) const {
      double x0;
      auto const& s = sp[fetch(x, x0)];
      return s[1] + x0 * (2.0 * s[2] + x0 * 3.0 * s[3]);
    }
    double fpp(double x) const {
      double x0;
      auto const& s = sp[fetch(x, x0)];
      return 2 * s[2] + 6.0 * x0 * s[3];
    }
  };

  // ---------------------------------------------------------------- DataEAM (data.cpp:37-153)

  struct DataEAM {
    std::size_t n = 0;
    double rcut = 0;
    std::vector<std::string> names;
    std::vector<double> mass;
    std::vector<Spline> F, phi, v;

    std::size_t index(std::size_t i, std::size_t j) const { return i + n * j; }
    std::size_t sym_index(std::size_t i, std::size_t j) const { return index(std::max(i, j), std::min(i, j)); }

    Spline const& f_of(std::uint32_t t) const { return F[t]; }
    Spline const& phi_of(std::uint32_t a, std::uint32_t b) const { return phi[index(a, b)]; }
    Spline const& v_of(std::uint32_t a, std::uint32_t b) const { return v[sym_index(a, b)]; }

    static std::istringstream line(std::ifstream& in) {
      std::string s;
      if (!std::getline(in, s)) throw Invalid("eam file terminated too soon");
      return std::istringstream{s};
    }

    static std::vector<double> chunked(std::ifstream& in, std::size_t cnt, std::size_t k) {
      std::vector<double> raw;
      raw.reserve(cnt);
      std::istringstream l;
      for (std::size_t i = 0; i < cnt; ++i) {
        if (i % k == 0) l = line(in);
        double t;
        l >> t;
        raw.push_back(t);
      }
      return raw;
    }

    explicit DataEAM(std::string const& path) {
      std::ifstream in(path);
      if (!in.good()) throw Invalid("could not open eam file");
      for (int i = 0; i < 3; ++i) line(in);
      {
        auto l = line(in);
        int nt;
        l >> nt;
        n = static_cast<std::size_t>(nt);
        for (std::size_t i = 0; i < n; ++i) {
          std::string s;
          l >> s;
          names.push_back(s);
        }
      }
      F.resize(n);
      phi.resize(n * n);
      v.resize(n * n);
      mass.resize(n);
      std::size_t numP, numR;
      double delP, delR;
      line(in) >> numP >> delP >> numR >> delR >> rcut;
      for (std::size_t i = 0; i < n; ++i) {
        std::size_t atomic;
        line(in) >> atomic >> mass[i];
        F[i] = Spline{chunked(in, numP, 5), delP};
        for (std::size_t j = 0; j < n; ++j) phi[index(i, j)] = Spline{chunked(in, numR, 5), delR};
      }
      for (std::size_t i = 0; i < n; ++i) {
        for (std::size_t j = 0; j <= i; ++j) {
          std::vector<double> raw = chunked(in, numR, 5);
          for (std::size_t k = 0; k < raw.size(); k++) raw[k] /= delR * static_cast<double>(k);
          raw[0] = raw[1];
          v[sym_index(i, j)] = Spline{std::move(raw), delR};
        }
      }
    }
  };

  // ---------------------------------------------------------------- Box + grid (orthorhombic only)

  struct Box {
    double L[3], invL[3];
    bool per[3];

    Box(double const* ext, int const* periodic) {
      for (int k = 0; k < 3; ++k) {
        if (!(ext[k] > 0)) throw Invalid("box extents must be positive");
        L[k] = ext[k];
        invL[k] = 1.0 / ext[k];
        per[k] = periodic[k] != 0;
      }
    }
    // orthorhombic.hpp:132-139
    void canon(double const* x, double* out) const {
      for (int k = 0; k < 3; ++k) out[k] = x[k] - L[k] * std::floor(x[k] * invL[k]);
    }
  };

  struct Grid {
    double rc;
    int shape[3], prod[3];
    double cell[3], inv_cell[3];

    // hypergrid.hpp:43-53
    Grid(Box const& b, double r_cut) : rc(r_cut) {
      if (!(r_cut > 0)) throw Invalid("r_cut must be positive");
      for (int k = 0; k < 3; ++k) {
        if (!(b.L[k] > r_cut)) throw Invalid("r_cut too large for box");
        shape[k] = 2 + static_cast<int>(b.L[k] / r_cut);
        cell[k] = b.L[k] / std::floor(b.L[k] / r_cut);
        inv_cell[k] = 1.0 / cell[k];
      }
      prod[0] = 1;
      prod[1] = shape[0];
      prod[2] = shape[0] * shape[1];
    }
    int ncells() const { return shape[0] * shape[1] * shape[2]; }
    // hypergrid.hpp:75-99
    int cell_idx(double const* x) const {
      int idx = 0;
      for (int k = 0; k < 3; ++k) {
        int i = static_cast<int>((x[k] + cell[k]) * inv_cell[k]);
        i = std::min(std::max(i, 0), shape[k] - 1);
        idx += i * prod[k];
      }
      return idx;
    }
  };

  // neigh/adjacent.hpp:40-70: adjacent cells in x-fastest order, excluding the cell itself.
  inline std::vector<std::vector<int>> adjacent_cells(Grid const& g) {
    std::vector<std::vector<int>> adj(static_cast<std::size_t>(g.ncells()));
    for (int cz = 0; cz < g.shape[2]; ++cz)
      for (int cy = 0; cy < g.shape[1]; ++cy)
        for (int cx = 0; cx < g.shape[0]; ++cx) {
          int c[3] = {cx, cy, cz};
          int beg[3], end[3];
          for (int k = 0; k < 3; ++k) {
            beg[k] = std::max(c[k] - 1, 0);
            end[k] = std::min(c[k] + 2, g.shape[k]);
          }
          int self = cx + cy * g.prod[1] + cz * g.prod[2];
          auto& out = adj[static_cast<std::size_t>(self)];
          for (int z = beg[2]; z < end[2]; ++z)
            for (int y = beg[1]; y < end[1]; ++y)
              for (int x = beg[0]; x < end[0]; ++x) {
                int m = x + y * g.prod[1] + z * g.prod[2];
                if (m != self) out.push_back(m);
              }
        }
    return adj;
  }

  // ---------------------------------------------------------------- List (list.cpp:37-165)

  struct List {
    static constexpr long MAX_GHOST_RATIO = 26;  // list.hpp:78
    static constexpr int NONE = std::numeric_limits<int>::max();

    Box box;
    Grid grid;
    std::vector<std::vector<int>> adj;
    long n = 0, n_plus_ghosts = 0;
    std::vector<double> r;     // 3 per slot (interleaved), real atoms then ghosts
    std::vector<long> image;   // real index of each slot
    std::vector<int> next, head;
    std::vector<std::vector<int>> nl;

    List(Box const& b, double r_cut) : box(b), grid(b, r_cut), adj(adjacent_cells(grid)) {}

    double const* pos(long s) const { return &r[static_cast<std::size_t>(3 * s)]; }

    void rebuild(double const* positions, long count, int threads) {
      if (threads <= 0) throw Invalid("threads must be positive");
      if (count != n) {
        n = count;
        r.assign(static_cast<std::size_t>(3 * n * (1 + MAX_GHOST_RATIO)), 0.0);
        image.assign(static_cast<std::size_t>(n * (1 + MAX_GHOST_RATIO)), 0);
        next.assign(image.size(), NONE);
        nl.assign(static_cast<std::size_t>(n), {});
        for (long i = 0; i < n; ++i) image[static_cast<std::size_t>(i)] = i;
      }
      for (long i = 0; i < n; ++i) box.canon(positions + 3 * i, &r[static_cast<std::size_t>(3 * i)]);
      make_ghosts();
      head.assign(static_cast<std::size_t>(grid.ncells()), NONE);
      for (long i = 0; i < n_plus_ghosts; ++i) {
        int c = grid.cell_idx(pos(i));
        next[static_cast<std::size_t>(i)] = head[static_cast<std::size_t>(c)];
        head[static_cast<std::size_t>(c)] = static_cast<int>(i);
      }
#pragma omp parallel for num_threads(threads) schedule(static)
      for (long i = 0; i < n; ++i) build(i);
    }

    // list.cpp:100-132: axis by axis, a plus pass then a minus pass over the slots that existed
    // before this axis was processed.
    void make_ghosts() {
      long slot = n;
      long const cap = n * (1 + MAX_GHOST_RATIO);
      for (int ax = 0; ax < 3; ++ax) {
        if (!box.per[ax]) continue;
        long const end = slot;
        for (int sign = 0; sign < 2; ++sign) {
          for (long j = 0; j < end; ++j) {
            double x[3] = {pos(j)[0], pos(j)[1], pos(j)[2]};
            bool make;
            if (sign == 0) {
              make = x[ax] < grid.rc;
              if (make) x[ax] += box.L[ax];
            } else {
              make = x[ax] > box.L[ax] - grid.rc;
              if (make) x[ax] -= box.L[ax];
            }
            if (make) {
              if (slot >= cap) throw std::length_error("ghost capacity");
              std::memcpy(&r[static_cast<std::size_t>(3 * slot)], x, sizeof x);
              image[static_cast<std::size_t>(slot)] = image[static_cast<std::size_t>(j)];
              ++slot;
            }
          }
        }
      }
      n_plus_ghosts = slot;
    }

    void build(long i) {
      auto& out = nl[static_cast<std::size_t>(i)];
      out.clear();
      double const* ri = pos(i);
      double const rc2 = grid.rc * grid.rc;
      int c = grid.cell_idx(ri);
      auto scan = [&](int cell, bool same) {
        for (int m = head[static_cast<std::size_t>(cell)]; m != NONE; m = next[static_cast<std::size_t>(m)]) {
          if (same && m == i) continue;
          double const* rm = pos(m);
          if (sq3(ri[0] - rm[0], ri[1] - rm[1], ri[2] - rm[2]) < rc2) out.push_back(m);
        }
      };
      scan(c, true);
      for (int a : adj[static_cast<std::size_t>(c)]) scan(a, false);
    }

    // list.cpp:37-51
    void update(double const* delta) {
      for (long i = 0; i < 3 * n; ++i) r[static_cast<std::size_t>(i)] -= delta[i];
      for (long s = n; s < n_plus_ghosts; ++s) {
        long im = image[static_cast<std::size_t>(s)];
        for (int k = 0; k < 3; ++k) r[static_cast<std::size_t>(3 * s + k)] -= delta[3 * im + k];
      }
    }

    // list.hpp:139-154
    template <typename F>
    void for_neighbours(long i, double r_cut, F&& f) const {
      if (r_cut > grid.rc) throw Invalid("r_cut bigger than the list cut-off");
      double const* ri = pos(i);
      for (int m : nl[static_cast<std::size_t>(i)]) {
        double const* rm = pos(m);
        double dr[3] = {rm[0] - ri[0], rm[1] - ri[1], rm[2] - ri[2]};
        double r_sq = sq3(dr[0], dr[1], dr[2]);
        if (r_sq < r_cut * r_cut) f(image[static_cast<std::size_t>(m)], std::sqrt(r_sq), dr);
      }
    }
  };

  // ---------------------------------------------------------------- EAM (eam.cpp:33-120)

  struct EAM {
    std::shared_ptr<DataEAM const> d;
    std::vector<double> fprime;

    double r_cut() const { return d->rcut; }

    // Runs body(i) for i in [0, n): a plain loop for one thread (so Spline::OutOfBounds propagates,
    // as eam.cpp:75-86 arranges), else an OpenMP static loop that re-throws the first exception.
    template <typename F>
    static void loop(long n, int threads, F&& body) {
      if (threads == 1) {
        for (long i = 0; i < n; ++i) body(i);
        return;
      }
      std::exception_ptr first;
#pragma omp parallel for num_threads(threads) schedule(static)
      for (long i = 0; i < n; ++i) {
        try {
          body(i);
        } catch (...) {
#pragma omp critical
          if (!first) first = std::current_exception();
        }
      }
      if (first) std::rethrow_exception(first);
    }

    double energy(std::uint32_t const* t, List const& nl, int threads) const {
      // eam.cpp:33-51 reduces v and F over threads; partial sums per atom are combined in index order
      // here so the result does not depend on the thread count.
      std::vector<double> vs(static_cast<std::size_t>(nl.n)), fs(static_cast<std::size_t>(nl.n));
      loop(nl.n, threads, [&](long a) {
        double rho = 0, v = 0;
        nl.for_neighbours(a, r_cut(), [&](long b, double r, double const*) {
          v += d->v_of(t[a], t[b]).f(r);
          rho += d->phi_of(t[b], t[a]).f(r);
        });
        vs[static_cast<std::size_t>(a)] = v;
        fs[static_cast<std::size_t>(a)] = d->f_of(t[a]).f(rho);
      });
      double v_sum = 0, f_sum = 0;
      for (long a = 0; a < nl.n; ++a) {
        v_sum += vs[static_cast<std::size_t>(a)];
        f_sum += fs[static_cast<std::size_t>(a)];
      }
      return (0.5 * v_sum) + f_sum;
    }

    void gradient(double* out, std::uint32_t const* t, std::uint8_t const* frozen, List const& nl, int threads) {
      fprime.resize(static_cast<std::size_t>(nl.n));
      loop(nl.n, threads, [&](long b) {
        double rho = 0;
        nl.for_neighbours(b, r_cut(), [&](long a, double r, double const*) { rho += d->phi_of(t[a], t[b]).f(r); });
        fprime[static_cast<std::size_t>(b)] = d->f_of(t[b]).fp(rho);
      });
      loop(nl.n, threads, [&](long g) {
        double grad[3] = {0, 0, 0};
        if (!frozen[g]) {
          nl.for_neighbours(g, r_cut(), [&](long a, double r, double const* dr) {
            double mag = d->v_of(t[a], t[g]).fp(r) + fprime[static_cast<std::size_t>(g)] * d->phi_of(t[a], t[g]).fp(r) +
                         fprime[static_cast<std::size_t>(a)] * d->phi_of(t[g], t[a]).fp(r);
            double s = mag / r;
            for (int k = 0; k < 3; ++k) grad[k] -= s * dr[k];
          });
        }
        for (int k = 0; k < 3; ++k) out[3 * g + k] = grad[k];
      });
    }
  };

  // EAM::hessian (src/potential/EAM/eam.cpp:122-233): the lower-triangular 3x3 blocks (a, z), a >= z,
  // of the dense 3n x 3n Hessian into out (row-major; rows of atom a), everything else zero; a frozen
  // atom's column and row blocks stay zero. Coefficients are formed in the order the reference's Eigen
  // expressions evaluate them (outer products (s u_r) w_c, sums left to right).
  inline void eam_hessian(EAM const& E, double* out, std::uint32_t const* t, std::uint8_t const* frozen, List const& nl,
                          int threads) {
    auto const& d = E.d;
    long const n = nl.n, N = 3 * n;
    std::fill(out, out + N * N, 0.0);
    std::vector<double> rho(static_cast<std::size_t>(n)), mu(static_cast<std::size_t>(3 * n));
    EAM::loop(n, threads, [&](long b) {  // rho and mu (A.13)
      double rb = 0, m[3] = {0, 0, 0};
      nl.for_neighbours(b, E.r_cut(), [&](long a, double r, double const* dr) {
        rb += d->phi_of(t[a], t[b]).f(r);
        double const fp = d->phi_of(t[a], t[b]).fp(r);
        for (int k = 0; k < 3; ++k) m[k] -= fp * dr[k] / r;
      });
      rho[static_cast<std::size_t>(b)] = rb;
      for (int k = 0; k < 3; ++k) mu[static_cast<std::size_t>(3 * b + k)] = m[k];
    });
    auto at = [&](long i, long j, int r, int c) -> double& { return out[(3 * i + r) * N + 3 * j + c]; };
    EAM::loop(n, threads, [&](long z) {  // column block z only
      if (frozen[z]) return;
      double const* v = &mu[static_cast<std::size_t>(3 * z)];
      double const fzpp = d->f_of(t[z]).fpp(rho[static_cast<std::size_t>(z)]);
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) at(z, z, r, c) = (fzpp * v[r]) * v[c];
      nl.for_neighbours(z, E.r_cut(), [&](long a, double r, double const* dr) {
        double const rho_z = rho[static_cast<std::size_t>(z)], rho_a = rho[static_cast<std::size_t>(a)];
        double const A = (d->v_of(t[a], t[z]).fp(r) + d->f_of(t[z]).fp(rho_z) * d->phi_of(t[a], t[z]).fp(r) +
                          d->f_of(t[a]).fp(rho_a) * d->phi_of(t[z], t[a]).fp(r)) /
                         r;
        double const B = d->v_of(t[a], t[z]).fpp(r) + d->f_of(t[z]).fp(rho_z) * d->phi_of(t[a], t[z]).fpp(r) +
                         d->f_of(t[a]).fp(rho_a) * d->phi_of(t[z], t[a]).fpp(r);
        double const pza = d->phi_of(t[z], t[a]).fp(r);
        double const ABFpp = (A - B - d->f_of(t[a]).fpp(rho_a) * (pza * pza)) / (r * r);
        for (int i = 0; i < 3; ++i)
          for (int c = 0; c < 3; ++c) at(z, z, i, c) += (i == c ? A : A * 0.0) - (ABFpp * dr[i]) * dr[c];
        if (a > z && !frozen[a]) {
          double const BArr = (B - A) / (r * r);
          double const ur = d->f_of(t[z]).fpp(rho_z) * d->phi_of(t[a], t[z]).fp(r) / r;
          double const ru = d->f_of(t[a]).fpp(rho_a) * d->phi_of(t[z], t[a]).fp(r) / r;
          double const* muz = &mu[static_cast<std::size_t>(3 * z)];
          double const* mua = &mu[static_cast<std::size_t>(3 * a)];
          for (int i = 0; i < 3; ++i)
            for (int c = 0; c < 3; ++c)
              at(a, z, i, c) += (((-BArr * dr[i]) * dr[c] - (i == c ? A : A * 0.0)) + (ur * dr[i]) * muz[c]) -
                                (ru * mua[i]) * dr[c];
        }
        double const ddFg = d->f_of(t[a]).fpp(rho_a) * d->phi_of(t[z], t[a]).fp(r);
        nl.for_neighbours(a, E.r_cut(), [&](long g, double r_ag, double const* dr_ag) {
          double const sx = dr[0] + dr_ag[0], sy = dr[1] + dr_ag[1], sz = dr[2] + dr_ag[2];
          if ((g > z && !frozen[g]) || (g == z && std::sqrt((sx * sx + sy * sy) + sz * sz) > 1e-6)) {
            double const mag = ddFg / (r * r_ag) * d->phi_of(t[g], t[a]).fp(r_ag);
            for (int i = 0; i < 3; ++i)
              for (int c = 0; c < 3; ++c) at(g, z, i, c) -= (mag * dr_ag[i]) * dr[c];
          }
        });
      });
    });
  }

  // ---------------------------------------------------------------- vector helpers (core.hpp:634-680)

  using Vec = std::vector<double>;

  inline double gdot(Vec const& a, Vec const& b) {
    double s = 0;
    for (std::size_t i = 0; i < a.size(); ++i) s += a[i] * b[i];
    return s;
  }
  inline double gnorm(Vec const& a) { return std::sqrt(gdot(a, a)); }

  // ---------------------------------------------------------------- StepLBFGS (lbfgs_core.cpp:29-87)

  struct StepLBFGS {
    int m;
    int k = 0;
    std::vector<Vec> s, y;
    std::vector<double> rho, alpha;
    Vec prev_x, prev_g, q, out;

    explicit StepLBFGS(int n) : m(n), s(static_cast<std::size_t>(n)), y(static_cast<std::size_t>(n)),
                                rho(static_cast<std::size_t>(n)), alpha(static_cast<std::size_t>(n)) {}

    void clear() { k = 0; }

    Vec& newton_step(Vec const& x, Vec const& g) {
      std::size_t const N = x.size();
      int prev = (k - 1) % m;
      if (k > 0) {
        if (prev_x.size() != N) throw Invalid("history size mismatch");
        auto& sp = s[static_cast<std::size_t>(prev)];
        auto& yp = y[static_cast<std::size_t>(prev)];
        sp.resize(N);
        yp.resize(N);
        for (std::size_t i = 0; i < N; ++i) {
          sp[i] = x[i] - prev_x[i];
          yp[i] = g[i] - prev_g[i];
        }
        rho[static_cast<std::size_t>(prev)] = 1.0 / std::abs(gdot(sp, yp));
      }
      prev_x = x;
      prev_g = g;
      q = g;
      int incur = k <= m ? 0 : k - m;
      int bound = k <= m ? k : m;
      for (int i = bound - 1; i >= 0; --i) {
        auto j = static_cast<std::size_t>((i + incur) % m);
        alpha[j] = rho[j] * gdot(s[j], q);
        for (std::size_t e = 0; e < N; ++e) q[e] -= alpha[j] * y[j][e];
      }
      out.resize(N);
      if (k > 0) {
        auto pp = static_cast<std::size_t>(prev);
        double scale = 1.0 / rho[pp] / gdot(y[pp], y[pp]);
        for (std::size_t e = 0; e < N; ++e) out[e] = q[e] * scale;
      } else {
        out = q;
      }
      for (int i = 0; i <= bound - 1; ++i) {
        auto j = static_cast<std::size_t>((i + incur) % m);
        double beta = rho[j] * gdot(y[j], out);
        for (std::size_t e = 0; e < N; ++e) out[e] += (alpha[j] - beta) * s[j][e];
      }
      ++k;
      return out;
    }
  };

  struct Potential {  // the three things the minimisers need from Generic (generic.hpp:79-115)
    EAM* eam;
    std::uint32_t const* types;
    std::uint8_t const* frozen;
    double r_cut() const { return eam->r_cut(); }
    void gradient(Vec& out, List const& nl) const {
      out.resize(static_cast<std::size_t>(3 * nl.n));
      eam->gradient(out.data(), types, frozen, nl, 1);
    }
    double energy(List const& nl) const { return eam->energy(types, nl, 1); }
  };

  inline double skin_of(double skin_frac, double r_cut) {
    return std::max(std::pow(skin_frac, 1. / 3.) - 1, 0.0) * r_cut;
  }

  // ---------------------------------------------------------------- LBFGS::minimise (lbfgs.cpp:29-115)

  struct LBFGSOptions {
    int n = 10, iter_max = 2000;
    double f2norm = 1e-6, skin_frac = 1.1, proj_tol = 0, max_trust = 0.5, min_trust = 0.01, grow_trust = 1.5,
           shrink_trust = 0.5;
  };

  // Returns true on failure (the reference's convention); *iters receives the steps taken.
  inline bool lbfgs_minimise(LBFGSOptions const& o, Box const& box, Potential const& pot, Vec& x, Vec& g, int* iters) {
    StepLBFGS core(o.n);
    double skin = skin_of(o.skin_frac, pot.r_cut());
    List nl(box, pot.r_cut() + skin);
    long const N = static_cast<long>(x.size() / 3);
    nl.rebuild(x.data(), N, 1);
    pot.gradient(g, nl);
    double trust = o.min_trust, acc = 0;
    for (int i = 0; i < o.iter_max; ++i) {
      if (iters) *iters = i;
      if (gdot(g, g) < o.f2norm * o.f2norm) return false;
      Vec& Hg = core.newton_step(x, g);
      double sc = std::min(1.0, trust / gnorm(Hg));
      for (double& e : Hg) e *= sc;
      acc += std::sqrt(gdot(Hg, Hg));
      for (std::size_t e = 0; e < x.size(); ++e) x[e] -= Hg[e];
      if (acc > 0.5 * skin) {
        nl.rebuild(x.data(), N, 1);
        acc = 0;
      } else {
        nl.update(Hg.data());
      }
      pot.gradient(g, nl);
      double proj = gdot(g, Hg);
      if (proj < -o.proj_tol) {
        trust = std::max(o.min_trust, o.shrink_trust * trust);
      } else if (proj > o.proj_tol) {
        trust = std::min(o.max_trust, o.grow_trust * trust);
      }
    }
    if (iters) *iters = o.iter_max;
    return true;
  }

  // ---------------------------------------------------------------- Rotor (rotor.cpp:33-164)

  struct RotorOptions {
    int n = 6, iter_max_rot = 20;
    double delta_r = 0.001, theta_tol = 1 * M_PI / 360.;
    bool relax_in_convex = true;
  };

  inline void trans_proj(Vec& x) {
    std::size_t const N = x.size() / 3;
    double p[3] = {0, 0, 0};
    for (std::size_t i = 0; i < N; ++i)
      for (int k = 0; k < 3; ++k) p[k] += x[3 * i + k];
    double inv = 1.0 / static_cast<double>(N);
    for (double& e : p) e *= inv;
    for (std::size_t i = 0; i < N; ++i)
      for (int k = 0; k < 3; ++k) x[3 * i + k] -= p[k];
  }

  struct Rotor {
    RotorOptions o;
    StepLBFGS core;
    Vec delta, delta_prev, axisp, g0, g1, g1p, dg;
    long grad_calls = 0;

    explicit Rotor(RotorOptions const& opt) : o(opt), core(opt.n) {}

    double r_cut(Potential const& pot) const { return pot.r_cut() + o.delta_r * 2; }

    double eff_gradient(Vec& out, Vec& axis, Potential const& pot, List& nl, int count_frozen) {
      std::size_t const N = axis.size();
      delta.assign(N, 0);
      delta_prev.assign(N, 0);
      axisp.assign(N, 0);
      dg.assign(N, 0);
      core.clear();
      pot.gradient(g0, nl);
      for (std::size_t e = 0; e < N; ++e) delta[e] = -o.delta_r * axis[e];
      nl.update(delta.data());
      std::swap(delta, delta_prev);
      pot.gradient(g1, nl);
      grad_calls += 2;
      Vec diff(N);
      double curv = [&] {
        for (int i = 0;; i++) {
          for (std::size_t e = 0; e < N; ++e) dg[e] = g1[e] - g0[e];
          double t = gdot(dg, axis);
          for (std::size_t e = 0; e < N; ++e) dg[e] -= t * axis[e];
          if (count_frozen == 0) trans_proj(dg);
          Vec& theta = core.newton_step(axis, dg);
          double tp = gdot(theta, axis);
          for (std::size_t e = 0; e < N; ++e) theta[e] -= tp * axis[e];
          double inv = 1 / gnorm(theta);
          for (double& e : theta) e *= inv;
          for (std::size_t e = 0; e < N; ++e) diff[e] = g1[e] - g0[e];
          double b_1 = gdot(diff, theta) / o.delta_r;
          double c_x0 = gdot(diff, axis) / o.delta_r;
          double theta_1 = -0.5 * std::atan(b_1 / std::abs(c_x0));
          if (std::abs(theta_1) < o.theta_tol || (i >= o.iter_max_rot && c_x0 < 0) || i > 10 * o.iter_max_rot) {
            return c_x0;
          }
          double c1 = std::cos(theta_1), s1 = std::sin(theta_1);
          for (std::size_t e = 0; e < N; ++e) axisp[e] = axis[e] * c1 + theta[e] * s1;
          for (std::size_t e = 0; e < N; ++e) delta[e] = -o.delta_r * axisp[e];
          std::swap(delta, delta_prev);
          for (std::size_t e = 0; e < N; ++e) delta[e] = delta_prev[e] - delta[e];
          nl.update(delta.data());
          pot.gradient(g1p, nl);
          ++grad_calls;
          for (std::size_t e = 0; e < N; ++e) diff[e] = g1p[e] - g0[e];
          double c_x1 = gdot(diff, axisp) / o.delta_r;
          double a_1 = (c_x0 - c_x1 + b_1 * std::sin(2 * theta_1)) / (1 - std::cos(2 * theta_1));
          double theta_min = 0.5 * std::atan(b_1 / a_1);
          if (a_1 * std::cos(2 * theta_min) - a_1 + b_1 * std::sin(2 * theta_min) > 0) theta_min += M_PI / 2;
          double cm = std::cos(theta_min), sm = std::sin(theta_min);
          for (std::size_t e = 0; e < N; ++e) axis[e] = axis[e] * cm + theta[e] * sm;
          double w1 = std::sin(theta_1 - theta_min) / std::sin(theta_1);
          double w1p = sm / std::sin(theta_1);
          double w0 = 1 - cm - sm * std::tan(0.5 * theta_1);
          for (std::size_t e = 0; e < N; ++e) g1[e] = w1 * g1[e] + w1p * g1p[e] + w0 * g0[e];
          if (std::abs(theta_min) < o.theta_tol) {
            for (std::size_t e = 0; e < N; ++e) diff[e] = g1[e] - g0[e];
            return gdot(diff, axis) / o.delta_r;
          }
        }
      }();
      for (std::size_t e = 0; e < N; ++e) delta[e] = -delta_prev[e];
      nl.update(delta.data());
      out.resize(N);
      double p = gdot(g0, axis);
      if (!o.relax_in_convex && curv > 0) {
        for (std::size_t e = 0; e < N; ++e) out[e] = -p * axis[e];
      } else {
        for (std::size_t e = 0; e < N; ++e) out[e] = g0[e] - 2 * p * axis[e];
      }
      if (count_frozen == 0) trans_proj(out);
      return curv;
    }
  };

  // ---------------------------------------------------------------- Dimer (dimer.cpp:28-171)

  struct DimerOptions {
    int n = 10, max_steps = 1000, hist_check_freq = 5;
    double f2norm = 1e-5, skin_frac = 1.1, proj_tol = 0, max_trust = 0.5, min_trust = 0.05, grow_trust = 1.5,
           shrink_trust = 0.5, convex_max = 3;
    bool use_history = true;
  };

  enum Exit : int { success = 0, convex = -1, iter_max = -2, collision = -3, uninit = -4 };

  struct DimerStats {
    int steps = 0;
    long grad_calls = 0;
    double curv = 0;
  };

  inline int dimer_find_sp(DimerOptions const& o, RotorOptions const& ro, Box const& box, Potential const& pot, Vec& x,
                           Vec& axis, Vec const& in_min, std::vector<Vec> const& hist_sp, double theta_tol,
                           int count_frozen, DimerStats* st) {
    StepLBFGS core(o.n);
    Rotor rotor(ro);
    double skin = skin_of(o.skin_frac, rotor.r_cut(pot));
    List nl(box, rotor.r_cut(pot) + skin);
    long const N = static_cast<long>(x.size() / 3);
    nl.rebuild(x.data(), N, 1);
    Vec eff;
    double curv = rotor.eff_gradient(eff, axis, pot, nl, count_frozen);
    double trust = o.min_trust, acc = 0, convex_count = 0;
    Vec d1(x.size()), d2(x.size());
    auto finish = [&](int code, int i) {
      if (st) {
        st->steps = i;
        st->grad_calls = rotor.grad_calls;
        st->curv = curv;
      }
      return code;
    };
    for (int i = 0; i < o.max_steps; ++i) {
      double mag_g = gdot(eff, eff);
      if (mag_g < o.f2norm * o.f2norm) return finish(success, i);
      if (convex_count >= o.convex_max) return finish(convex, i);
      if (o.use_history && i % o.hist_check_freq == 0) {
        double ctheta = -1;
        for (auto const& sp : hist_sp) {
          for (std::size_t e = 0; e < x.size(); ++e) {
            d1[e] = x[e] - in_min[e];
            d2[e] = sp[e] - in_min[e];
          }
          double dt = gdot(d1, d2);
          double sn = gnorm(d2);
          double on = gnorm(d1);
          ctheta = std::max(ctheta, dt / (sn * on));
          if (ctheta > std::cos(theta_tol)) return finish(collision, i);
        }
      }
      Vec& Hg = core.newton_step(x, eff);
      double sc = std::min(1.0, trust / gnorm(Hg));
      for (double& e : Hg) e *= sc;
      acc += std::sqrt(gdot(Hg, Hg));
      for (std::size_t e = 0; e < x.size(); ++e) x[e] -= Hg[e];
      if (acc > 0.5 * skin) {
        nl.rebuild(x.data(), N, 1);
        acc = 0;
      } else {
        nl.update(Hg.data());
      }
      curv = rotor.eff_gradient(eff, axis, pot, nl, count_frozen);
      convex_count = curv > 0 ? convex_count + 1 : 0;
      double proj = gdot(eff, Hg);
      if (proj < -o.proj_tol) {
        trust = std::max(o.min_trust, o.shrink_trust * trust);
      } else if (proj > o.proj_tol) {
        trust = std::min(o.max_trust, o.grow_trust * trust);
      }
    }
    return finish(iter_max, o.max_steps);
  }

  // ---------------------------------------------------------------- Xoshiro256** (random.hpp:42-162)

  // A UniformRandomBitGenerator (random.hpp:42-162), so std::normal_distribution draws from it exactly
  // as the reference's Master::perturb does (find.cpp:1150-1164).
  struct Xoshiro {
    using result_type = std::uint64_t;
    static constexpr result_type min() { return 0; }
    static constexpr result_type max() { return std::numeric_limits<result_type>::max(); }
    std::uint64_t s[4];
    static std::uint64_t rotl(std::uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    std::uint64_t operator()() {
      std::uint64_t const res = rotl(s[1] * 5, 7) * 9;
      std::uint64_t const t = s[1] << 17;
      s[2] ^= s[0];
      s[3] ^= s[1];
      s[1] ^= s[2];
      s[0] ^= s[3];
      s[2] ^= t;
      s[3] = rotl(s[3], 45);
      return res;
    }
  };

}  // namespace orc

// ==================================================================== C ABI for the test harness

namespace {
  template <typename F>
  int guarded(F&& f) {
    try {
      f();
      return orc::OK;
    } catch (orc::OutOfBounds const&) {
      return orc::SPLINE_OOB;
    } catch (std::length_error const&) {
      return orc::GHOST_OVERFLOW;
    } catch (...) {
      return orc::INVALID;
    }
  }

  struct Handle {
    std::shared_ptr<orc::DataEAM const> data;
  };
}  // namespace

extern "C" {

// Dimer + Rotor options, field order as in dimer.hpp:56-98 then rotor.hpp:47-60.
struct orc_dimer_options {
  int n, max_steps, hist_check_freq, use_history;
  double f2norm, skin_frac, proj_tol, max_trust, min_trust, grow_trust, shrink_trust, convex_max;
  int rot_n, iter_max_rot, relax_in_convex, pad_;
  double delta_r, theta_tol;
};

// LBFGS options, lbfgs.hpp:56-80.
struct orc_lbfgs_options {
  int n, iter_max;
  double f2norm, skin_frac, proj_tol, max_trust, min_trust, grow_trust, shrink_trust;
};

void* orc_eam_load(char const* path) {
  try {
    return new Handle{std::make_shared<orc::DataEAM const>(std::string(path))};
  } catch (...) {
    return nullptr;
  }
}

void orc_eam_free(void* h) { delete static_cast<Handle*>(h); }

double orc_eam_rcut(void* h) { return static_cast<Handle*>(h)->data->rcut; }

int orc_eam_ntypes(void* h) { return static_cast<int>(static_cast<Handle*>(h)->data->n); }

double orc_eam_mass(void* h, int t) { return static_cast<Handle*>(h)->data->mass[static_cast<std::size_t>(t)]; }

// kind 0 = F(type a), 1 = phi(a, b), 2 = v(a, b); deriv 0/1/2 = f/fp/fpp.
int orc_spline_eval(void* h, int kind, int a, int b, int deriv, double x, double* out) {
  auto const& d = *static_cast<Handle*>(h)->data;
  return guarded([&] {
    orc::Spline const& s = kind == 0 ? d.f_of(static_cast<std::uint32_t>(a))
                          : kind == 1 ? d.phi_of(static_cast<std::uint32_t>(a), static_cast<std::uint32_t>(b))
                                      : d.v_of(static_cast<std::uint32_t>(a), static_cast<std::uint32_t>(b));
    *out = deriv == 0 ? s.f(x) : deriv == 1 ? s.fp(x) : s.fpp(x);
  });
}

// Spline coefficient table (n_spines x 4) of one function, for byte-level comparison.
long orc_spline_table(void* h, int kind, int a, int b, double* out, long cap) {
  auto const& d = *static_cast<Handle*>(h)->data;
  orc::Spline const& s = kind == 0 ? d.f_of(static_cast<std::uint32_t>(a))
                        : kind == 1 ? d.phi_of(static_cast<std::uint32_t>(a), static_cast<std::uint32_t>(b))
                                    : d.v_of(static_cast<std::uint32_t>(a), static_cast<std::uint32_t>(b));
  long n = static_cast<long>(s.sp.size());
  if (out && cap >= 4 * n) std::memcpy(out, s.sp.data(), sizeof(double) * 4 * static_cast<std::size_t>(n));
  return n;
}

// Spline::Spline (spline.cpp:27-103) of an arbitrary table: coefficients, and f / fp / fpp at points.
long orc_spline_build(double const* y, long n, double dx, double* out, long cap) {
  orc::Spline s(std::vector<double>(y, y + n), dx);
  long const count = static_cast<long>(s.sp.size());
  if (out && cap >= 4 * count) std::memcpy(out, s.sp.data(), sizeof(double) * 4 * static_cast<std::size_t>(count));
  return count;
}

int orc_spline_points(double const* y, long n, double dx, double const* x, long m, double* out) {
  return guarded([&] {
    orc::Spline s(std::vector<double>(y, y + n), dx);
    for (long k = 0; k < m; ++k) {
      out[3 * k + 0] = s.f(x[k]);
      out[3 * k + 1] = s.fp(x[k]);
      out[3 * k + 2] = s.fpp(x[k]);
    }
  });
}

void* orc_list_new(double const* ext, int const* periodic, double r_cut) {
  try {
    return new orc::List(orc::Box(ext, periodic), r_cut);
  } catch (...) {
    return nullptr;
  }
}

void orc_list_free(void* l) { delete static_cast<orc::List*>(l); }

int orc_list_rebuild(void* l, double const* pos, long n, int threads) {
  return guarded([&] { static_cast<orc::List*>(l)->rebuild(pos, n, threads); });
}

int orc_list_update(void* l, double const* delta) {
  return guarded([&] { static_cast<orc::List*>(l)->update(delta); });
}

long orc_list_num_ghosts(void* l) {
  auto* L = static_cast<orc::List*>(l);
  return L->n_plus_ghosts - L->n;
}

// Grid shape (3 ints) of the list.
void orc_list_shape(void* l, int* shape) {
  auto* L = static_cast<orc::List*>(l);
  for (int k = 0; k < 3; ++k) shape[k] = L->grid.shape[k];
}

// Positions (3 per slot) and real index of every real + ghost slot.
long orc_list_slots(void* l, double* pos, long* image, long cap) {
  auto* L = static_cast<orc::List*>(l);
  if (cap >= L->n_plus_ghosts) {
    std::memcpy(pos, L->r.data(), sizeof(double) * 3 * static_cast<std::size_t>(L->n_plus_ghosts));
    std::memcpy(image, L->image.data(), sizeof(long) * static_cast<std::size_t>(L->n_plus_ghosts));
  }
  return L->n_plus_ghosts;
}

// Neighbours of every atom within r_cut, in for_neighbours order: counts[n], then CSR (real index,
// dr xyz). Returns the total, or -1 on error; fills idx/dr only if total <= cap.
long orc_list_neighbours(void* l, double r_cut, int* counts, int* idx, double* dr, long cap) {
  auto* L = static_cast<orc::List*>(l);
  long total = 0;
  try {
    for (long i = 0; i < L->n; ++i) {
      int c = 0;
      L->for_neighbours(i, r_cut, [&](long m, double, double const* d) {
        if (total < cap) {
          idx[total] = static_cast<int>(m);
          for (int k = 0; k < 3; ++k) dr[3 * total + k] = d[k];
        }
        ++total;
        ++c;
      });
      counts[i] = c;
    }
  } catch (...) {
    return -1;
  }
  return total;
}

// Raw slot lists (real or ghost slot ids) in list order, CSR as above. For order checks.
long orc_list_raw(void* l, int* counts, int* slots, long cap) {
  auto* L = static_cast<orc::List*>(l);
  long total = 0;
  for (long i = 0; i < L->n; ++i) {
    auto const& v = L->nl[static_cast<std::size_t>(i)];
    counts[i] = static_cast<int>(v.size());
    for (int m : v) {
      if (total < cap) slots[total] = m;
      ++total;
    }
  }
  return total;
}

int orc_eam_energy(void* h, void* l, std::uint32_t const* types, int threads, double* e) {
  return guarded([&] {
    orc::EAM eam{static_cast<Handle*>(h)->data, {}};
    *e = eam.energy(types, *static_cast<orc::List*>(l), threads);
  });
}

int orc_eam_gradient(void* h, void* l, std::uint32_t const* types, std::uint8_t const* frozen, int threads, double* g) {
  return guarded([&] {
    orc::EAM eam{static_cast<Handle*>(h)->data, {}};
    eam.gradient(g, types, frozen, *static_cast<orc::List*>(l), threads);
  });
}

// EAM::hessian (eam.cpp:122-233) as a dense row-major 3n x 3n lower-block-triangular matrix.
int orc_eam_hessian(void* h, void* l, std::uint32_t const* types, std::uint8_t const* frozen, int threads, double* out) {
  return guarded([&] {
    orc::EAM eam{static_cast<Handle*>(h)->data, {}};
    orc::eam_hessian(eam, out, types, frozen, *static_cast<orc::List*>(l), threads);
  });
}

// Per-atom embedding derivative F'(rho) of the last density pass (for intermediate parity checks).
int orc_eam_fprime(void* h, void* l, std::uint32_t const* types, std::uint8_t const* frozen, double* fp) {
  return guarded([&] {
    auto* L = static_cast<orc::List*>(l);
    orc::EAM eam{static_cast<Handle*>(h)->data, {}};
    std::vector<double> g(static_cast<std::size_t>(3 * L->n));
    eam.gradient(g.data(), types, frozen, *L, 1);
    std::memcpy(fp, eam.fprime.data(), sizeof(double) * static_cast<std::size_t>(L->n));
  });
}

// O(N^2) brute-force minimum-image neighbour count (tests/neigh/list.cpp:42-97): for each i the
// sorted real indices j with |min-image(r_j - r_i)|^2 < r_cut^2. Fills CSR; returns total.
long orc_brute_neighbours(double const* ext, int const* periodic, double const* pos, long n, double r_cut, int* counts,
                          int* idx, double* dr, long cap) {
  std::vector<std::array<double, 3>> disps;
  for (int sz = -1; sz <= 1; ++sz)
    for (int sy = -1; sy <= 1; ++sy)
      for (int sx = -1; sx <= 1; ++sx) {
        int s[3] = {sx, sy, sz};
        std::array<double, 3> off{0, 0, 0};
        bool zero = true, all0 = (sx == 0 && sy == 0 && sz == 0);
        for (int k = 0; k < 3; ++k)
          if (periodic[k]) {
            off[static_cast<std::size_t>(k)] += ext[k] * s[k];
            if (s[k] != 0) zero = false;
          }
        if (all0 || !zero) disps.push_back(off);
      }
  long total = 0;
  for (long i = 0; i < n; ++i) {
    int c = 0;
    for (long j = 0; j < n; ++j) {
      if (i == j) continue;
      double best[3] = {std::numeric_limits<double>::max(), 0, 0};
      double bestn = std::numeric_limits<double>::infinity();
      for (auto const& d : disps) {
        double v[3];
        for (int k = 0; k < 3; ++k) v[k] = (pos[3 * j + k] + d[static_cast<std::size_t>(k)]) - pos[3 * i + k];
        double nn = std::sqrt(orc::sq3(v[0], v[1], v[2]));
        if (nn < bestn) {
          bestn = nn;
          std::memcpy(best, v, sizeof v);
        }
      }
      if (orc::sq3(best[0], best[1], best[2]) < r_cut * r_cut) {
        if (total < cap) {
          idx[total] = static_cast<int>(j);
          for (int k = 0; k < 3; ++k) dr[3 * total + k] = best[k];
        }
        ++total;
        ++c;
      }
    }
    counts[i] = c;
  }
  return total;
}

// LBFGS::minimise on positions x (3N, in/out); g receives the final gradient. Returns status;
// *failed = the reference's bool (true = not converged), *iters = steps taken.
int orc_lbfgs_minimise(void* h, orc_lbfgs_options const* opt, double const* ext, int const* periodic, long n,
                       double* x, std::uint32_t const* types, std::uint8_t const* frozen, double* g, int* failed,
                       int* iters) {
  return guarded([&] {
    orc::EAM eam{static_cast<Handle*>(h)->data, {}};
    orc::Potential pot{&eam, types, frozen};
    orc::LBFGSOptions o;
    o.n = opt->n;
    o.iter_max = opt->iter_max;
    o.f2norm = opt->f2norm;
    o.skin_frac = opt->skin_frac;
    o.proj_tol = opt->proj_tol;
    o.max_trust = opt->max_trust;
    o.min_trust = opt->min_trust;
    o.grow_trust = opt->grow_trust;
    o.shrink_trust = opt->shrink_trust;
    orc::Vec X(x, x + 3 * n), G;
    *failed = orc::lbfgs_minimise(o, orc::Box(ext, periodic), pot, X, G, iters) ? 1 : 0;
    std::memcpy(x, X.data(), sizeof(double) * X.size());
    std::memcpy(g, G.data(), sizeof(double) * G.size());
  });
}

// Dimer::find_sp. x/axis (3N) in/out; in_min (3N); hist (n_hist x 3N). Writes the exit code,
// translation steps, gradient evaluations and final curvature.
int orc_dimer_find_sp(void* h, orc_dimer_options const* opt, double const* ext, int const* periodic, long n,
                      double* x, double* axis, std::uint32_t const* types, std::uint8_t const* frozen,
                      double const* in_min, double const* hist, int n_hist, double theta_tol, int count_frozen,
                      int* exit_code, int* steps, long* grad_calls, double* curv) {
  return guarded([&] {
    orc::EAM eam{static_cast<Handle*>(h)->data, {}};
    orc::Potential pot{&eam, types, frozen};
    orc::DimerOptions o;
    o.n = opt->n;
    o.max_steps = opt->max_steps;
    o.hist_check_freq = opt->hist_check_freq;
    o.use_history = opt->use_history != 0;
    o.f2norm = opt->f2norm;
    o.skin_frac = opt->skin_frac;
    o.proj_tol = opt->proj_tol;
    o.max_trust = opt->max_trust;
    o.min_trust = opt->min_trust;
    o.grow_trust = opt->grow_trust;
    o.shrink_trust = opt->shrink_trust;
    o.convex_max = opt->convex_max;
    orc::RotorOptions ro;
    ro.n = opt->rot_n;
    ro.iter_max_rot = opt->iter_max_rot;
    ro.delta_r = opt->delta_r;
    ro.theta_tol = opt->theta_tol;
    ro.relax_in_convex = opt->relax_in_convex != 0;
    std::size_t const M = static_cast<std::size_t>(3 * n);
    orc::Vec X(x, x + M), A(axis, axis + M), IM(in_min, in_min + M);
    std::vector<orc::Vec> H;
    for (int k = 0; k < n_hist; ++k) H.emplace_back(hist + static_cast<std::size_t>(k) * M, hist + (static_cast<std::size_t>(k) + 1) * M);
    orc::DimerStats st;
    *exit_code = orc::dimer_find_sp(o, ro, orc::Box(ext, periodic), pot, X, A, IM, H, theta_tol, count_frozen, &st);
    *steps = st.steps;
    *grad_calls = st.grad_calls;
    *curv = st.curv;
    std::memcpy(x, X.data(), sizeof(double) * M);
    std::memcpy(axis, A.data(), sizeof(double) * M);
  });
}

// Many independent dimer searches spread over threads, one search per thread at a time, as
// Master::find_batch does (find.cpp:697-732, inner num_threads = 1 at find.cpp:990). Searches are
// packed: offsets[s]..offsets[s+1] are the atoms of search s; ext (3 per search), periodic (3 per
// search). Exit codes land in exit_codes[s]. Returns the first non-ok status.
int orc_dimer_batch(void* h, orc_dimer_options const* opt, int n_search, long const* offsets, double const* ext,
                    int const* periodic, double* x, double* axis, std::uint32_t const* types,
                    std::uint8_t const* frozen, int const* count_frozen, int threads, int* exit_codes, int* steps) {
  int worst = orc::OK;
#pragma omp parallel for num_threads(threads) schedule(dynamic, 1)
  for (int s = 0; s < n_search; ++s) {
    long o0 = offsets[s], n = offsets[s + 1] - offsets[s];
    long gc;
    double cv;
    int st = orc_dimer_find_sp(h, opt, ext + 3 * s, periodic + 3 * s, n, x + 3 * o0, axis + 3 * o0, types + o0,
                               frozen + o0, x + 3 * o0, nullptr, 0, 0.0, count_frozen[s], exit_codes + s, steps + s,
                               &gc, &cv);
    if (st != orc::OK) {
#pragma omp critical
      worst = worst == orc::OK ? st : worst;
    }
  }
  return worst;
}

// xoshiro256** stream (random.hpp:42-162) for fixtures: fills out[n] with raw 64-bit outputs.
void orc_xoshiro(std::uint64_t const* seed, std::uint64_t* out, long n) {
  orc::Xoshiro g{{seed[0], seed[1], seed[2], seed[3]}};
  for (long i = 0; i < n; ++i) out[i] = g();
}

// count draws of one libstdc++ std::normal_distribution<double>(mean, stddev) from the stream seeded by
// state (updated in place).
void orc_normal_draws(std::uint64_t* state, double mean, double stddev, long count, double* out) {
  orc::Xoshiro g{{state[0], state[1], state[2], state[3]}};
  std::normal_distribution<double> d(mean, stddev);
  for (long i = 0; i < count; ++i) out[i] = d(g);
  std::memcpy(state, g.s, sizeof g.s);
}

// Master::perturb (src/saddle/find.cpp:1147-1214) with the oracle's List (built with cut-off r_pert on
// in_pos, find.cpp:217-219): the stddev prime draws, then per unfrozen neighbour of the centre in
// for_neighbours order three position draws (scaled by 1 - r / r_pert) and three axis draws, then the
// centre's, the axis normalised over all 3n (sequential sum). state is updated in place.
int orc_perturb(void* l, long centre, double const* in_pos, std::uint8_t const* frozen, long n, double stddev_opt,
                double r_pert, std::uint64_t* state, double* out_pos, double* out_axis, double* stddev_used) {
  return guarded([&] {
    auto const& nl = *static_cast<orc::List*>(l);
    orc::Xoshiro prng{{state[0], state[1], state[2], state[3]}};
    std::normal_distribution<double> normal(0., 1.);
    std::normal_distribution<double> prime(stddev_opt, stddev_opt / 3.0);
    double stddev = -1;
    while (stddev < 0) stddev = prime(prng);
    std::normal_distribution<double> gauss(0, stddev);
    std::memcpy(out_pos, in_pos, sizeof(double) * 3 * static_cast<std::size_t>(n));
    std::fill_n(out_axis, 3 * n, 0.0);
    nl.for_neighbours(centre, r_pert, [&](long a, double r, double const*) {
      if (!frozen[a]) {
        double const env = 1. - r / r_pert;
        for (int k = 0; k < 3; ++k) out_pos[3 * a + k] += gauss(prng) * env;
        for (int k = 0; k < 3; ++k) out_axis[3 * a + k] += normal(prng);
      }
    });
    for (int k = 0; k < 3; ++k) out_pos[3 * centre + k] += gauss(prng);
    for (int k = 0; k < 3; ++k) out_axis[3 * centre + k] += normal(prng);
    double ss = 0;
    for (long k = 0; k < 3 * n; ++k) ss += out_axis[k] * out_axis[k];
    double const nrm = std::sqrt(ss);
    for (long k = 0; k < 3 * n; ++k) out_axis[k] /= nrm;
    *stddev_used = stddev;
    std::memcpy(state, prng.s, sizeof prng.s);
  });
}

int orc_max_threads() { return omp_get_max_threads(); }

// AdjacentCells (neigh/adjacent.hpp:40-70) of one cell of a grid of the given shape; returns the count.
int orc_adjacent(int const* shape, int cell, int* out) {
  orc::Grid g(orc::Box(std::array<double, 3>{10, 10, 10}.data(), std::array<int, 3>{0, 0, 0}.data()), 1.0);
  for (int k = 0; k < 3; ++k) g.shape[k] = shape[k];
  g.prod[0] = 1;
  g.prod[1] = shape[0];
  g.prod[2] = shape[0] * shape[1];
  auto adj = orc::adjacent_cells(g);
  auto const& v = adj[static_cast<std::size_t>(cell)];
  std::copy(v.begin(), v.end(), out);
  return static_cast<int>(v.size());
}

// HyperGrid(extents, r_cut).cell_idx(x) (system/boxes/hypergrid.hpp:43-99).
int orc_cell_idx(double const* ext, double r_cut, double const* x) {
  int const per[3] = {0, 0, 0};
  orc::Grid g(orc::Box(ext, per), r_cut);
  return g.cell_idx(x);
}

}  // extern "C"
