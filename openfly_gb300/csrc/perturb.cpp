// perturb.cpp -- Master::perturb (src/saddle/find.cpp:1147-1214) with the reference's random stream.
//
// The reference draws from a per-thread xoshiro256** 1.0 generator (include/libfly/utility/random.hpp:
// 42-162) through std::normal_distribution. Reproducing its draws needs three pieces, restated here
// from their published definitions:
//   * xoshiro256** 1.0 (Blackman and Vigna): result = rotl(s1 * 5, 7) * 9, then the xor/shift/rotate
//     state update; long_jump advances the stream by 2^192 outputs (the reference seeds thread k's
//     generator k long jumps after thread 0's, find.cpp:188-193);
//   * a uniform double in [0, 1) from one 64-bit output: (double)x / 2^64, clamped below 1 (the
//     canonical-real construction libstdc++ uses for a 64-bit engine and a 53-bit mantissa);
//   * normal variates by Marsaglia's polar method as libstdc++ arranges it: draw u, v = 2U - 1 until
//     0 < s = u^2 + v^2 <= 1, m = sqrt(-2 ln s / s), return v m and keep u m for the next call of the
//     same distribution object; each object scales by its stddev and adds its mean.
// perturb keeps the reference's draw order: the stddev prime draws (repeated while negative), then per
// neighbour of the centre within r_pert, in List::for_neighbours order, three position draws and three
// axis draws (from two distribution objects with separate cached values), then the centre's three and
// three. This unit is compiled with -ffp-contract=off, like the reference's binary64 arithmetic.

#include <cmath>
#include <cstring>
#include <limits>
#include <vector>

#include "internal.hpp"

namespace flygpu {

  namespace {

    std::uint64_t rotl(std::uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }

    std::uint64_t xoshiro_next(flygpu_xoshiro& g) {
      std::uint64_t* s = g.s;
      std::uint64_t const out = rotl(s[1] * 5, 7) * 9;
      std::uint64_t const t = s[1] << 17;
      s[2] ^= s[0];
      s[3] ^= s[1];
      s[1] ^= s[2];
      s[0] ^= s[3];
      s[2] ^= t;
      s[3] = rotl(s[3], 45);
      return out;
    }

    void xoshiro_jump(flygpu_xoshiro& g, std::uint64_t const (&poly)[4]) {
      std::uint64_t acc[4] = {0, 0, 0, 0};
      for (std::uint64_t word : poly)
        for (int b = 0; b < 64; ++b) {
          if (word & (std::uint64_t{1} << b))
            for (int k = 0; k < 4; ++k) acc[k] ^= g.s[k];
          xoshiro_next(g);
        }
      std::memcpy(g.s, acc, sizeof acc);
    }

    // Uniform double in [0, 1) from one output.
    double canonical(flygpu_xoshiro& g) {
      double const r = static_cast<double>(xoshiro_next(g)) / 18446744073709551616.0;  // 2^64
      return r >= 1.0 ? std::nextafter(1.0, 0.0) : r;
    }

    // One normal distribution object: mean, stddev and its cached second value.
    struct Normal {
      double mean, stddev;
      bool have = false;
      double saved = 0;
      double operator()(flygpu_xoshiro& g) {
        double z;
        if (have) {
          have = false;
          z = saved;
        } else {
          double u, v, s;
          do {
            u = 2.0 * canonical(g) - 1.0;
            v = 2.0 * canonical(g) - 1.0;
            s = u * u + v * v;
          } while (s > 1.0 || s == 0.0);
          double const m = std::sqrt(-2 * std::log(s) / s);
          saved = u * m;
          have = true;
          z = v * m;
        }
        return z * stddev + mean;
      }
    };

  }  // namespace

  double perturb(std::vector<int> const& nbr, std::vector<double> const& nbr_r, std::int64_t centre,
                 double const* in_pos, std::uint8_t const* frozen, std::int64_t n, double stddev_opt, double r_pert,
                 flygpu_xoshiro& g, double* out_pos, double* out_axis) {
    Normal normal{0.0, 1.0};
    Normal prime{stddev_opt, stddev_opt / 3.0};
    double stddev = -1;
    while (stddev < 0) stddev = prime(g);
    Normal gauss{0.0, stddev};
    std::memcpy(out_pos, in_pos, sizeof(double) * 3 * static_cast<std::size_t>(n));
    std::fill_n(out_axis, 3 * n, 0.0);
    for (std::size_t k = 0; k < nbr.size(); ++k) {
      std::int64_t const a = nbr[k];
      if (frozen[a]) continue;
      double const env = 1. - nbr_r[k] / r_pert;
      for (int c = 0; c < 3; ++c) out_pos[3 * a + c] += gauss(g) * env;
      for (int c = 0; c < 3; ++c) out_axis[3 * a + c] += normal(g);
    }
    for (int c = 0; c < 3; ++c) out_pos[3 * centre + c] += gauss(g);
    for (int c = 0; c < 3; ++c) out_axis[3 * centre + c] += normal(g);
    double ss = 0;
    for (std::int64_t k = 0; k < 3 * n; ++k) ss += out_axis[k] * out_axis[k];
    double const norm = std::sqrt(ss);
    for (std::int64_t k = 0; k < 3 * n; ++k) out_axis[k] /= norm;
    return stddev;
  }

}  // namespace flygpu

extern "C" {

int flygpu_xoshiro_seed(flygpu_xoshiro* g, const uint64_t seed[4]) {
  if (!g || !seed) return FLYGPU_INVALID_ARG;
  if ((seed[0] | seed[1] | seed[2] | seed[3]) == 0) {
    flygpu::set_error("xoshiro256**: an all-zero seed is invalid");
    return FLYGPU_INVALID_ARG;
  }
  std::memcpy(g->s, seed, sizeof g->s);
  return FLYGPU_OK;
}

uint64_t flygpu_xoshiro_next(flygpu_xoshiro* g) { return flygpu::xoshiro_next(*g); }

void flygpu_xoshiro_long_jump(flygpu_xoshiro* g) {
  static constexpr std::uint64_t poly[4] = {0x76e15d3efefdcbbfULL, 0xc5004e441c522fb3ULL, 0x77710069854ee241ULL,
                                            0x39109bb02acbe635ULL};
  flygpu::xoshiro_jump(*g, poly);
}

int flygpu_normal_draws(flygpu_xoshiro* g, double mean, double stddev, int64_t count, double* out) {
  if (!g || count < 0 || (count > 0 && !out)) return FLYGPU_INVALID_ARG;
  flygpu::Normal d{mean, stddev};
  for (int64_t k = 0; k < count; ++k) out[k] = d(*g);
  return FLYGPU_OK;
}

}  // extern "C"
