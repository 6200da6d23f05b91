// Host build of the engine's hand-written exponentials (dfloat.cuh / physics.cuh
// compiled with BGB_HOST_EMULATION: the same operation sequence with IEEE
// round-to-nearest host arithmetic) measured against long-double references.
// Prints one "name max_relative_error" line per routine.
#define BGB_HOST_EMULATION
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "../bear_gb300/csrc/physics.cuh"

using namespace bgb;

int main() {
  std::mt19937_64 g(20261203);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  double e_exp2 = 0, e_tang2048 = 0, e_pow10 = 0, e_planck = 0, e_expneg = 0, ulp2048 = 0;
  double e_tang2048f = 0, ulp2048f = 0, e_negdf_scaled = 0, ulp_negdf = 0;
  for (int i = 0; i < 2000000; ++i) {
    // double-float 2^y over the exponent range of the opacity terms
    const double y = -140.0 + 180.0 * U(g);
    const df2 yd = df_from_double(y);
    int n;
    const df2 m = df_exp2(yd, n, kExp2TabHi, kExp2TabLo);
    const long double ry = exp2l((long double)yd.hi + (long double)yd.lo);
    e_exp2 = std::fmax(e_exp2, (double)fabsl(((long double)m.hi + m.lo) * exp2l(n) / ry - 1));
    // FP64 exp(x), x in [-700, 0] (the recurrence's exp(-delta)), with thin layers oversampled
    double x = -700.0 * U(g);
    if (i % 4 == 0) x = -1e-3 * U(g);
    const long double rx = expl((long double)x);
    const double b = exp_tang2048(x, kExp2TabD2048);
    e_tang2048 = std::fmax(e_tang2048, (double)fabsl(b / rx - 1));
    const double rd = (double)rx;
    ulp2048 = std::fmax(ulp2048, (double)fabsl(((long double)b - rx) / (std::nextafter(rd, 1e308) - rd)));
    // the same with the table index from a float estimate of x (the kernels' d2f_trunc of -x)
    const double bf = exp_tang2048_f(x, -d2f_trunc(-x), kExp2TabD2048);
    e_tang2048f = std::fmax(e_tang2048f, (double)fabsl(bf / rx - 1));
    if (x >= -40.0)  // a >= 4e-18: the range where a's last bits can reach the intensities
      ulp2048f = std::fmax(ulp2048f, (double)fabsl(((long double)bf - rx) / (std::nextafter(rd, 1e308) - rd)));
    // exp(-d) in FP64 from a double-float d (the recurrence's a = exp(-tau/mu)), against the
    // exact exponential of the double-float input: the reduction rounds its low part once, an
    // error ~1e-14 d relative (about what d carries as a double-float product); thin layers, where
    // a - 1 is what matters, are oversampled and held to the ulp
    {
      double xd = 40.0 * U(g);
      if (i % 3 == 0) xd = 1e-3 * U(g);
      if (i % 7 == 0) xd = 40.0 + 660.0 * U(g);
      const df2 dd = df_from_double(xd);
      const double ad = exp_neg_df(dd, kExp2TabD2048);
      const long double ra = expl(-((long double)dd.hi + (long double)dd.lo));
      const double rel = (double)fabsl(ad / ra - 1);
      e_negdf_scaled = std::fmax(e_negdf_scaled, rel / std::fmax(xd, 1.0));
      if (xd < 1e-3) {
        const double rr = (double)ra;
        ulp_negdf = std::fmax(ulp_negdf, (double)fabsl(((long double)ad - ra) / (std::nextafter(rr, 1e308) - rr)));
      }
    }
    // double-float exp(-d) of the adjoint
    const double d = 60.0 * U(g);
    const df2 en = df_exp_neg(df_from_double(d), kExp2TabHi, kExp2TabLo);
    const long double rn = expl(-(long double)(double)df_from_double(d).hi - (long double)df_from_double(d).lo);
    e_expneg = std::fmax(e_expneg, (double)fabsl(((long double)en.hi + en.lo) / rn - 1));
  }
  for (int i = 0; i < 1000000; ++i) {
    // 10^x for log10 cross sections
    const double x = -40.0 + 30.0 * U(g);
    const df2 xd = df_from_double(x);
    int n;
    const df2 m = df_exp2(df_mul(xd, df2{kLog2_10Hi, kLog2_10Lo}), n, kExp2TabHi, kExp2TabLo);
    const long double r = powl(10.0L, (long double)xd.hi + (long double)xd.lo);
    e_pow10 = std::fmax(e_pow10, (double)fabsl(((long double)m.hi + m.lo) * exp2l(n) / r - 1));
    // Planck function c1 / (exp(c2 / T) - 1), nu in [1000, 26000] cm^-1, T in [50, 4000] K
    const double nu = 1000.0 + 25000.0 * U(g), T = 50.0 + 3950.0 * U(g);
    const double c1 = 2.0 * 6.62606896e-27 * 2.99792458e10 * 2.99792458e10 * nu * nu * nu;
    const double c2 = 6.62606896e-27 * nu * 2.99792458e10 / 1.3806504e-16;
    const long double rp = (long double)c1 / expm1l((long double)c2 / T);
    const double c2l = c2 * 1.4426950408889634;
    const df2 c2ld = {(float)c2l, (float)(c2l - (double)(float)c2l)};
    const double Bp = planck_df(df_from_double(c1), c2ld, df_from_double(1.0 / T), kExp2TabHi, kExp2TabLo);
    if (c2 / T < 690.0) e_planck = std::fmax(e_planck, (double)fabsl(Bp / rp - 1));
  }
  // integer-pipe conversions: bit-identical to the FP64 conversions they replace
  long long conv_mismatch = 0;
  std::uniform_int_distribution<unsigned> bits(0u, 0xffffffffu);
  auto same = [](double a, double b) {
    return (std::isnan(a) && std::isnan(b)) || bgb_double_as_ll(a) == bgb_double_as_ll(b);
  };
  for (int i = 0; i < 4000000; ++i) {
    unsigned u = bits(g);
    if (i < 512) u = (i & 1) ? (0x80000000u | (unsigned)(i >> 1)) : (unsigned)(i >> 1);  // zeros, subnormals
    if (i >= 512 && i < 1024) u = ((unsigned)(i & 255) << 23) | (u & 0x807fffffu);        // every exponent
    float f;
    std::memcpy(&f, &u, 4);
    if (!same(f2d_bits(f), (double)f)) ++conv_mismatch;
  }
  for (int k = -3000000; k <= 3000000; ++k)
    if (!same(i2d_bits(k), (double)k)) ++conv_mismatch;
  for (int k : {2147483647, -2147483647, 1 << 30, -(1 << 30)})
    if (!same(i2d_bits(k), (double)k)) ++conv_mismatch;
  // df_exp2 outside the clamp: 2^y underflows / overflows in the callers, NaN propagates
  long long edge_bad = 0;
  for (float yv : {-1e30f, -1e6f, -20000.0f, 20000.0f, 1e6f, 1e30f, -INFINITY, INFINITY}) {
    int n;
    const df2 m = df_exp2(df2{yv, 0.0f}, n, kExp2TabHi, kExp2TabLo);
    const double v = ((double)m.hi + m.lo) * std::ldexp(1.0, std::max(-1100, std::min(1100, n)));
    if (!std::isfinite(m.hi) || (yv < 0 && v != 0.0) || (yv > 0 && !std::isinf(v))) ++edge_bad;
  }
  {
    int n;
    const df2 m = df_exp2(df2{NAN, 0.0f}, n, kExp2TabHi, kExp2TabLo);
    if (!std::isnan(m.hi)) ++edge_bad;
  }
  // df_recip over the ranges of 1/tau and 1/(1 - u) (host: correctly rounded float
  // reciprocal; the device's approximate one is within 2^-23, which the Newton step with
  // its square term absorbs)
  double e_recip = 0;
  for (int i = 0; i < 1000000; ++i) {
    const double b = std::ldexp(1.0 + U(g), (int)(180.0 * U(g)) - 90);
    const df2 bd = df_from_double(b);
    const df2 r = df_recip(bd);
    const long double ref = 1.0L / ((long double)bd.hi + bd.lo);
    e_recip = std::fmax(e_recip, (double)fabsl(((long double)r.hi + r.lo) / ref - 1));
  }
  // df_from_double_bits: within 2^-48 of the value in its range, df_from_double outside it
  double e_split = 0;
  long long split_fallback_bad = 0;
  for (int i = 0; i < 2000000; ++i) {
    double x = std::ldexp(1.0 + U(g), (int)(200.0 * U(g)) - 100);
    if (i & 1) x = -x;
    if (i % 1000 == 0) x = 0.0;
    const df2 d = df_from_double_bits(x);
    const int ex = std::ilogb(x);
    if (x == 0.0 || ex < -60 || ex >= 101) {
      const df2 r = df_from_double(x);
      if (bgb_float_as_uint(d.hi) != bgb_float_as_uint(r.hi) || bgb_float_as_uint(d.lo) != bgb_float_as_uint(r.lo))
        ++split_fallback_bad;
    } else {
      e_split = std::fmax(e_split, (double)fabsl(((long double)d.hi + d.lo) / (long double)x - 1));
      if (std::fabs(d.lo) >= std::ldexp(std::fabs(d.hi), -23)) ++split_fallback_bad;
    }
  }
  // d2f_trunc: below the float range 0, else within 2^-23 of the value
  double e_trunc = 0;
  for (int i = 0; i < 1000000; ++i) {
    const double d = std::ldexp(U(g), (int)(277.0 * U(g)) - 150);  // up to 2^127
    const float f = d2f_trunc(d);
    if (d < std::ldexp(1.0, -126)) e_trunc = std::fmax(e_trunc, f == 0.0f ? 0.0 : 1.0);
    else e_trunc = std::fmax(e_trunc, std::fabs((double)f / d - 1));
  }
  std::printf("df_exp2 %.3e\nexp_tang2048 %.3e\nexp_tang2048_ulp %.3f\ndf_exp_neg %.3e\n"
              "df_pow10 %.3e\nplanck_df %.3e\nconversion_mismatches %lld\nexp_tang2048_f %.3e\n"
              "exp_tang2048_f_ulp %.3f\nd2f_trunc %.3e\ndf_exp2_edge_failures %lld\ndf_recip %.3e\n"
              "df_from_double_bits %.3e\ndf_from_double_bits_failures %lld\n"
              "exp_neg_df_per_d %.3e\nexp_neg_df_thin_ulp %.3f\n",
              e_exp2, e_tang2048, ulp2048, e_expneg, e_pow10, e_planck, conv_mismatch, e_tang2048f,
              ulp2048f, e_trunc, edge_bad, e_recip, e_split, split_fallback_bad, e_negdf_scaled, ulp_negdf);
  return 0;
}
