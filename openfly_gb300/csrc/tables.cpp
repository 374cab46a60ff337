// tables.cpp -- host side of the EAM tables: LAMMPS eam/fs parsing and natural cubic splines.
//
// Parsing follows DataEAM::DataEAM (src/potential/EAM/data.cpp:67-153): three comment lines, a types
// line, a grid line "numP dP numR dR rcut", then per type a header line, F (numP values) and
// phi(i, j) for every j (numR values each, stored at i + n*j, data.hpp:109-112), then r*v for every
// j <= i (divided by r = k*dR with raw[0] = raw[1], data.cpp:133-151). Splines follow
// Spline::Spline (src/utility/spline.cpp:27-103). This unit is compiled with -ffp-contract=off so the
// binary64 coefficients are the reference's, bit for bit, on any host.

#include <algorithm>
#include <cmath>
#include <fstream>
#include <memory>
#include <sstream>

#include "internal.hpp"

namespace flygpu {

  int spline_spines(std::size_t n_samples) { return static_cast<int>(n_samples + 5 - 1); }

  void build_spline(std::vector<double> y, double dx, double* out4, int n_spines) {
    double const last = y.back();
    for (int i = 0; i < 5; i++) y.push_back(last);
    std::size_t const n = y.size() - 1;
    if (static_cast<int>(n) != n_spines) fail(FLYGPU_INVALID_ARG, "spline size mismatch");
    std::vector<double> const& a = y;
    std::vector<double> b(n), d(n), alpha(n), c(n + 1), l(n + 1), mu(n + 1), z(n + 1);
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
      std::size_t const j = n - i;
      c[j] = z[j] - mu[j] * c[j + 1];
      b[j] = (a[j + 1] - a[j]) / dx - dx * (c[j + 1] + 2 * c[j]) / 3;
      d[j] = (c[j + 1] - c[j]) / (3 * dx);
    }
    for (std::size_t i = 0; i < n; ++i) {
      out4[4 * i + 0] = a[i];
      out4[4 * i + 1] = b[i];
      out4[4 * i + 2] = c[i];
      out4[4 * i + 3] = d[i];
    }
  }

  namespace {

    std::istringstream next_line(std::ifstream& in) {
      std::string s;
      if (!std::getline(in, s)) fail(FLYGPU_INVALID_ARG, "eam file terminated too soon");
      return std::istringstream{s};
    }

    std::vector<double> read_chunked(std::ifstream& in, std::size_t count, std::size_t per_line) {
      std::vector<double> raw;
      raw.reserve(count);
      std::istringstream line;
      for (std::size_t i = 0; i < count; ++i) {
        if (i % per_line == 0) line = next_line(in);
        double t = 0;
        line >> t;
        raw.push_back(t);
      }
      return raw;
    }

    // Binary32 coefficients of every interval in its unit coordinate.
    std::vector<float4> unit32(SplineSet const& s) {
      std::size_t const total = static_cast<std::size_t>(s.count) * static_cast<std::size_t>(s.n_spines);
      std::vector<float4> f32(total);
      for (std::size_t k = 0; k < total; ++k) {
        double const* c = &s.host[4 * k];
        double const dx = s.dx;
        f32[k] = make_float4(static_cast<float>(c[0]), static_cast<float>(c[1] * dx),
                             static_cast<float>(c[2] * dx * dx), static_cast<float>(c[3] * dx * dx * dx));
      }
      return f32;
    }

    // Derivative coefficients of interval k in the unit coordinate: {b_hi, b_lo, 2c, 3d} with b = b dx,
    // c = c dx^2, d = d dx^3 formed in binary64 and b split into a binary32 pair.
    float4 unit_deriv32(SplineSet const& s, std::size_t k) {
      double const* c = &s.host[4 * k];
      double const dx = s.dx;
      double const b = c[1] * dx;
      float const bh = static_cast<float>(b);
      return make_float4(bh, static_cast<float>(b - static_cast<double>(bh)), static_cast<float>(2 * c[2] * dx * dx),
                         static_cast<float>(3 * c[3] * dx * dx * dx));
    }

    void upload(SplineSet& s) {
      std::size_t const total = static_cast<std::size_t>(s.count) * static_cast<std::size_t>(s.n_spines);
      std::vector<float4> const f32 = unit32(s);
      s.d64.reserve(total);
      s.d32.reserve(total);
      FLY_CUDA(cudaMemcpy(s.d64.p, s.host.data(), total * sizeof(D4), cudaMemcpyHostToDevice));
      FLY_CUDA(cudaMemcpy(s.d32.p, f32.data(), total * sizeof(float4), cudaMemcpyHostToDevice));
    }

  }  // namespace

}  // namespace flygpu

flygpu::TablesView flygpu_eam::view() const {
  flygpu::TablesView t{};
  t.n_types = n_types;
  t.nP = F.n_spines;
  t.nR = phi.n_spines;
  t.dP = F.dx;
  t.inv_dP = F.inv_dx;
  t.dR = phi.dx;
  t.inv_dR = phi.inv_dx;
  t.fdP = static_cast<float>(F.dx);
  t.finv_dP = static_cast<float>(F.inv_dx);
  t.fdR = static_cast<float>(phi.dx);
  t.finv_dR = static_cast<float>(phi.inv_dx);
  t.finv_dR_lo = static_cast<float>(phi.inv_dx - static_cast<double>(t.finv_dR));
  t.F64 = F.d64.p;
  t.phi64 = phi.d64.p;
  t.v64 = v.d64.p;
  t.F32 = F.d32.p;
  t.phi32 = phi.d32.p;
  t.v32 = v.d32.p;
  t.pv32 = pv.p;
  t.dv32 = dv.p;
  return t;
}

namespace flygpu {

  flygpu_eam* eam_load(char const* path) {
    std::ifstream in(path);
    if (!in.good()) fail(FLYGPU_INVALID_ARG, std::string("could not open eam file ") + path);
    auto E = std::make_unique<flygpu_eam>();
    for (int i = 0; i < 3; ++i) next_line(in);
    std::size_t n = 0;
    {
      auto line = next_line(in);
      int nt = 0;
      line >> nt;
      if (nt <= 0) fail(FLYGPU_INVALID_ARG, "eam file declares no types");
      n = static_cast<std::size_t>(nt);
      for (std::size_t i = 0; i < n; ++i) {
        std::string s;
        line >> s;
        E->names.push_back(s);
      }
    }
    std::size_t numP = 0, numR = 0;
    double delP = 0, delR = 0;
    next_line(in) >> numP >> delP >> numR >> delR >> E->r_cut;
    if (numP < 2 || numR < 2 || !(delP > 0) || !(delR > 0)) fail(FLYGPU_INVALID_ARG, "bad eam grid line");
    E->n_types = static_cast<int>(n);
    E->mass.resize(n);
    auto init = [](SplineSet& s, int count, std::size_t samples, double dx) {
      s.count = count;
      s.n_spines = spline_spines(samples);
      s.dx = dx;
      s.inv_dx = 1 / dx;
      s.host.assign(static_cast<std::size_t>(count) * static_cast<std::size_t>(s.n_spines) * 4, 0.0);
    };
    init(E->F, static_cast<int>(n), numP, delP);
    init(E->phi, static_cast<int>(n * n), numR, delR);
    init(E->v, static_cast<int>(n * n), numR, delR);
    auto slot = [](SplineSet& s, std::size_t k) { return &s.host[k * static_cast<std::size_t>(s.n_spines) * 4]; };
    for (std::size_t i = 0; i < n; ++i) {
      std::size_t atomic = 0;
      next_line(in) >> atomic >> E->mass[i];
      build_spline(read_chunked(in, numP, 5), delP, slot(E->F, i), E->F.n_spines);
      for (std::size_t j = 0; j < n; ++j) build_spline(read_chunked(in, numR, 5), delR, slot(E->phi, i + n * j), E->phi.n_spines);
    }
    for (std::size_t i = 0; i < n; ++i) {
      for (std::size_t j = 0; j <= i; ++j) {
        std::vector<double> raw = read_chunked(in, numR, 5);
        for (std::size_t k = 0; k < raw.size(); k++) raw[k] /= delR * static_cast<double>(k);
        raw[0] = raw[1];
        build_spline(raw, delR, slot(E->v, i + n * j), E->v.n_spines);
        if (i != j) std::copy_n(slot(E->v, i + n * j), static_cast<std::size_t>(E->v.n_spines) * 4, slot(E->v, j + n * i));
      }
    }
    upload(E->F);
    upload(E->phi);
    upload(E->v);
    {
      // merged records: [t_i][t_n][interval] = {phi[t_n + n t_i], v[t_i + n t_n]}
      int const nt = E->n_types;
      std::size_t const nR = static_cast<std::size_t>(E->phi.n_spines);
      std::vector<float4> const p32 = unit32(E->phi), v32 = unit32(E->v);
      std::vector<PairRec> rec(static_cast<std::size_t>(nt) * static_cast<std::size_t>(nt) * nR);
      for (int ti = 0; ti < nt; ++ti)
        for (int tn = 0; tn < nt; ++tn)
          for (std::size_t i = 0; i < nR; ++i) {
            PairRec& r = rec[(static_cast<std::size_t>(ti) * nt + tn) * nR + i];
            r.phi = p32[(static_cast<std::size_t>(tn) + static_cast<std::size_t>(nt) * ti) * nR + i];
            r.v = v32[(static_cast<std::size_t>(ti) + static_cast<std::size_t>(nt) * tn) * nR + i];
          }
      E->pv.reserve(rec.size());
      FLY_CUDA(cudaMemcpy(E->pv.p, rec.data(), rec.size() * sizeof(PairRec), cudaMemcpyHostToDevice));
      std::vector<DerRec> der(rec.size());
      for (int ti = 0; ti < nt; ++ti)
        for (int tn = 0; tn < nt; ++tn)
          for (std::size_t i = 0; i < nR; ++i) {
            DerRec& r = der[(static_cast<std::size_t>(ti) * nt + tn) * nR + i];
            r.v = unit_deriv32(E->v, (static_cast<std::size_t>(ti) + static_cast<std::size_t>(nt) * tn) * nR + i);
            r.phi = unit_deriv32(E->phi, (static_cast<std::size_t>(tn) + static_cast<std::size_t>(nt) * ti) * nR + i);
          }
      E->dv.reserve(der.size());
      FLY_CUDA(cudaMemcpy(E->dv.p, der.data(), der.size() * sizeof(DerRec), cudaMemcpyHostToDevice));
    }
    return E.release();
  }

}  // namespace flygpu
