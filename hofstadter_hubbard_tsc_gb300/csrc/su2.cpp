// Wigner 6j symbols in doubled-integer arguments (Racah single-sum formula).
// Same definition as W6JS of the reference (code/update.f90:1665-1716); the
// values are memoised per plan build in a hash map, the reference memoises them
// in fixed tables (code/pubdata.f90:16-23).
#include <cmath>
#include <mutex>
#include <unordered_map>
#include <cstdint>

namespace hh {

static double g_fact[302];
static std::once_flag g_fact_once;

static void init_fact() {
  g_fact[0] = 1.0;
  for (int i = 1; i < 302; ++i) g_fact[i] = g_fact[i - 1] * double(i);
}

static inline bool tri_ok(int a, int b, int c) {
  return c <= a + b && c >= std::abs(a - b) && ((a + b + c) & 1) == 0;
}

static inline double delta(int a, int b, int c) {
  return g_fact[(a + b - c) / 2] * g_fact[(a - b + c) / 2] * g_fact[(-a + b + c) / 2] /
         g_fact[(a + b + c) / 2 + 1];
}

static double w6j_eval(int j1, int j2, int j3, int l1, int l2, int l3) {
  if (j1 < 0 || j2 < 0 || j3 < 0 || l1 < 0 || l2 < 0 || l3 < 0) return 0.0;
  if (!tri_ok(j1, j2, j3) || !tri_ok(j1, l2, l3) || !tri_ok(l1, j2, l3) || !tri_ok(l1, l2, j3))
    return 0.0;
  const int a1 = j1 + j2 + j3, a2 = j1 + l2 + l3, a3 = l1 + j2 + l3, a4 = l1 + l2 + j3;
  const int b1 = j1 + j2 + l1 + l2, b2 = j2 + j3 + l2 + l3, b3 = j3 + j1 + l3 + l1;
  int tmin = a1;
  if (a2 > tmin) tmin = a2;
  if (a3 > tmin) tmin = a3;
  if (a4 > tmin) tmin = a4;
  int tmax = b1;
  if (b2 < tmax) tmax = b2;
  if (b3 < tmax) tmax = b3;
  if (tmax / 2 + 1 > 301) return std::nan("");
  double s = 0.0;
  for (int t = tmin; t <= tmax; t += 2) {
    double den = g_fact[(t - a1) / 2] * g_fact[(t - a2) / 2] * g_fact[(t - a3) / 2] *
                 g_fact[(t - a4) / 2] * g_fact[(b1 - t) / 2] * g_fact[(b2 - t) / 2] *
                 g_fact[(b3 - t) / 2];
    double term = g_fact[t / 2 + 1] / den;
    if ((t / 2) & 1) term = -term;
    s += term;
  }
  return s * std::sqrt(delta(j1, j2, j3) * delta(j1, l2, l3) * delta(l1, j2, l3) * delta(l1, l2, j3));
}

// Wigner 3j symbol (j1 j2 j3; m1 m2 m3), doubled arguments, by Racah's
// single-sum formula.  Every half-sum below is exact: the triangle and
// projection parities make each numerator even.
double w3j(int j1, int j2, int j3, int m1, int m2, int m3) {
  std::call_once(g_fact_once, init_fact);
  if (m1 + m2 + m3 != 0 || j1 < 0 || j2 < 0 || j3 < 0 || !tri_ok(j1, j2, j3)) return 0.0;
  if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0;
  if (((j1 - m1) & 1) || ((j2 - m2) & 1) || ((j3 - m3) & 1)) return 0.0;
  if ((j1 + j2 + j3) / 2 + 1 > 301) return std::nan("");
  int kmin = 0;
  if ((j2 - j3 - m1) / 2 > kmin) kmin = (j2 - j3 - m1) / 2;
  if ((j1 - j3 + m2) / 2 > kmin) kmin = (j1 - j3 + m2) / 2;
  int kmax = (j1 + j2 - j3) / 2;
  if ((j1 - m1) / 2 < kmax) kmax = (j1 - m1) / 2;
  if ((j2 + m2) / 2 < kmax) kmax = (j2 + m2) / 2;
  double s = 0.0;
  for (int k = kmin; k <= kmax; ++k) {
    double den = g_fact[k] * g_fact[(j1 + j2 - j3) / 2 - k] * g_fact[(j1 - m1) / 2 - k] *
                 g_fact[(j2 + m2) / 2 - k] * g_fact[(j3 - j2 + m1) / 2 + k] * g_fact[(j3 - j1 - m2) / 2 + k];
    s += (k & 1 ? -1.0 : 1.0) / den;
  }
  double pre = std::sqrt(delta(j1, j2, j3) * g_fact[(j1 + m1) / 2] * g_fact[(j1 - m1) / 2] * g_fact[(j2 + m2) / 2] *
                         g_fact[(j2 - m2) / 2] * g_fact[(j3 + m3) / 2] * g_fact[(j3 - m3) / 2]);
  return (((j1 - j2 - m3) / 2) & 1 ? -1.0 : 1.0) * pre * s;
}

double w6j(int j1, int j2, int j3, int l1, int l2, int l3) {
  std::call_once(g_fact_once, init_fact);
  static thread_local std::unordered_map<uint64_t, double> memo;
  if ((j1 | j2 | j3 | l1 | l2 | l3) >= 1024 || j1 < 0 || j2 < 0 || j3 < 0 || l1 < 0 || l2 < 0 ||
      l3 < 0)
    return w6j_eval(j1, j2, j3, l1, l2, l3);
  uint64_t k = (uint64_t(j1) << 50) | (uint64_t(j2) << 40) | (uint64_t(j3) << 30) |
               (uint64_t(l1) << 20) | (uint64_t(l2) << 10) | uint64_t(l3);
  auto it = memo.find(k);
  if (it != memo.end()) return it->second;
  double v = w6j_eval(j1, j2, j3, l1, l2, l3);
  memo.emplace(k, v);
  return v;
}

}  // namespace hh
