// Host restatement of the integer steps of exact_view_sum (spim_registration_gb300/csrc/inputs.cu),
// checked against IEEE double sums on random weight sets built to hit the edge cases: zeros,
// -0, denormals, tiny and large values, exponents spread past the certified range.  Every set
// the integer steps certify must give exactly (float)sum and (float)(sum - (float)sum) of the
// sequential double sum 0.0 + w_0 + w_1 + ...  The device function itself is checked bit for
// bit against the oracle by tests/test_gpu_inputs.py.
//
// usage: exact_view_sum_check <cases> <seed>; prints "cases C certified K mismatches M" and
// exits non-zero on any mismatch.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>

static unsigned bits_of(float f) {
  unsigned u;
  std::memcpy(&u, &f, 4);
  return u;
}
static float float_of(unsigned u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
static int clz64(long long k) { return k == 0 ? 64 : __builtin_clzll((unsigned long long)k); }

// k >= 0 rounded to `bits` significant bits, ties to even
static long long round_sig(long long k, int bits) {
  const int nb = 64 - clz64(k);
  if (nb <= bits) return k;
  const int sh = nb - bits;
  const long long low = k & ((1LL << sh) - 1), half = 1LL << (sh - 1);
  k -= low;
  if (low > half || (low == half && ((k >> sh) & 1))) k += 1LL << sh;
  return k;
}

// k * 2^e rounded once to float; false when not a normal float
static bool scaled_float(long long k, int e, float& out) {
  if (k == 0) {
    out = 0.f;
    return true;
  }
  const unsigned sign = k < 0 ? 0x80000000u : 0u;
  const long long a = round_sig(k < 0 ? -k : k, 24);
  const int nb = 64 - clz64(a);
  const unsigned m = nb >= 24 ? (unsigned)(a >> (nb - 24)) : (unsigned)a << (24 - nb);
  const int ex = nb - 1 + e + 127;
  if (ex < 1 || ex > 254) return false;
  out = float_of(sign | ((unsigned)ex << 23) | (m & 0x7fffffu));
  return true;
}

static bool exact_view_sum(const float* wv, int nv, float& hi, float& lo) {
  int emin = 1 << 20, emax = -(1 << 20);
  for (int v = 0; v < nv; ++v) {
    const unsigned b = bits_of(wv[v]);
    if (b & 0x80000000u) {
      if (b != 0x80000000u) return false;
      continue;
    }
    const int be = (int)(b >> 23);
    if (be == 255) return false;
    if (b == 0) continue;
    const int sv = (be ? be : 1) - 150;
    emin = std::min(emin, sv);
    emax = std::max(emax, sv);
  }
  if (emax < emin) {
    hi = lo = 0.f;
    return true;
  }
  if (emax - emin > 34) return false;
  long long k = 0;
  for (int v = 0; v < nv; ++v) {
    const unsigned b = bits_of(wv[v]);
    if (b == 0u || b == 0x80000000u) continue;
    const int be = (int)(b >> 23);
    const long long m = (long long)((b & 0x7fffffu) | (be ? 0x800000u : 0u));
    k = round_sig(k + (m << (((be ? be : 1) - 150) - emin)), 53);
  }
  const long long khi = round_sig(k, 24);
  return scaled_float(khi, emin, hi) && scaled_float(k - khi, emin, lo);
}

int main(int argc, char** argv) {
  const long long cases = argc > 1 ? std::atoll(argv[1]) : 1000000;
  std::mt19937_64 g(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 7);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  long long certified = 0, bad = 0;
  for (long long t = 0; t < cases; ++t) {
    const int nv = 1 + (int)(g() % 16);
    float w[16];
    for (int v = 0; v < nv; ++v) {
      const double u = U(g);
      switch (g() % 10) {
        case 0: w[v] = 0.f; break;
        case 1: w[v] = -0.f; break;
        case 2: w[v] = (float)u; break;
        case 3: w[v] = (float)(u * u * u * u); break;
        case 4: w[v] = (float)std::ldexp(u, -(int)(g() % 40)); break;
        case 5: w[v] = float_of((unsigned)(g() % 0x800000u)); break;  // denormal
        case 6: w[v] = (float)std::ldexp(1.0 + u, (int)(g() % 60) - 30); break;
        case 7: w[v] = (float)std::ldexp(u, (int)(g() % 20)); break;
        case 8: w[v] = 1.f; break;
        default: w[v] = float_of(bits_of((float)u) + (unsigned)(g() % 3)); break;
      }
    }
    float hi, lo;
    if (!exact_view_sum(w, nv, hi, lo)) continue;
    ++certified;
    volatile double s = 0.0;  // one IEEE double addition per view, in order
    for (int v = 0; v < nv; ++v) s = s + (double)w[v];
    const float rh = (float)s, rl = (float)(s - (double)rh);
    if (bits_of(rh) != bits_of(hi) || bits_of(rl) != bits_of(lo)) {
      if (bad < 5) std::printf("mismatch: nv=%d hi %a vs %a, lo %a vs %a\n", nv, hi, rh, lo, rl);
      ++bad;
    }
  }
  std::printf("cases %lld certified %lld mismatches %lld\n", cases, certified, bad);
  return bad != 0;
}
