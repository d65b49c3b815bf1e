// Host restatement of the FP64-free steps of blend_weight (spim_registration_gb300/csrc/inputs.cu),
// checked against the reference's double arithmetic (BlendingRealRandomAccess.java:44-121):
//  1. the lookup index: Math.round(relDist * 1000.0) for a float relDist in [0, 1), found by
//     two FMA sign tests around a first guess, against floor(double(rel) * 1000 + 0.5);
//  2. minDistance *= lookUp[i]: the certified float-pair product against
//     (float)((double)w * lookUp[i]) (a double product rounded to double, then to float).
// The table is filled as the reference fills it (d += 0.001 from 0 while d <= 1.0001).  Build
// with -ffp-contract=off: the restatement's separate multiplies and adds must not fuse.
//
// usage: blend_weight_check <cases> <seed>; prints "index C mismatches M product P certified K
// mismatches N" and exits non-zero on any mismatch.
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

struct FF {
  float hi, lo;
};

static bool round_pair(FF x, float& y) {
  y = x.hi + x.lo;
  if (x.hi == 0.f && x.lo == 0.f) return true;
  const unsigned b = bits_of(y);
  const unsigned ex = b & 0x7f800000u;
  if (ex <= (24u << 23) || ex == 0x7f800000u) return false;
  if (x.lo == 0.f) return true;
  if ((b & 0x007fffffu) == 0u) return false;
  const float half_ulp = float_of(ex - (24u << 23));
  const float d = (x.hi - y) + x.lo;
  return std::fabs(d) < half_ulp * 0.99993896484375f;
}

static FF ff_mul(FF a, FF b) {
  const float p = a.hi * b.hi;
  const float e = std::fmaf(a.hi, b.hi, -p);
  return {p, e + (a.hi * b.lo + a.lo * b.hi)};
}

static int lookup_index(float rel) {
  int idx = (int)std::floor(std::fmaf(rel, 1000.f, 0.5f));
  if (std::fmaf(rel, 1000.f, 0.5f - (float)idx) < 0.f)
    --idx;
  else if (std::fmaf(rel, 1000.f, -0.5f - (float)idx) >= 0.f)
    ++idx;
  return idx < 0 ? 0 : (idx > 1000 ? 1000 : idx);
}

int main(int argc, char** argv) {
  const long long cases = argc > 1 ? std::atoll(argv[1]) : 1000000;
  std::mt19937_64 g(argc > 2 ? std::strtoull(argv[2], nullptr, 10) : 7);
  std::uniform_real_distribution<double> U(0.0, 1.0);
  double lut[1001] = {};
  for (double d = 0; d <= 1.0001; d = d + 0.001) lut[(int)std::floor(d * 1000.0 + 0.5)] = (std::cos((1 - d) * M_PI) + 1) / 2;
  float lhi[1001], llo[1001];
  for (int k = 0; k <= 1000; ++k) {
    lhi[k] = (float)lut[k];
    llo[k] = (float)(lut[k] - (double)lhi[k]);
  }
  long long bad_idx = 0, certified = 0, bad_prod = 0;
  for (long long t = 0; t < cases; ++t) {
    // 1. index: generic floats, and dist / blending quotients beside the half steps
    float rel;
    if (t & 1) {
      rel = (float)U(g);
    } else {
      const float blend = (float)(1.0 + 999.0 * U(g));
      const float dist = (float)((double)(g() % 1000) + 0.5) * (blend / 1000.f);
      rel = dist / blend;
      const int nudge = (int)(g() % 5) - 2;  // a few ulps either way
      rel = float_of(bits_of(rel) + nudge);
    }
    if (rel >= 0.f && rel < 1.f) {
      const int want = (int)std::floor((double)rel * 1000.0 + 0.5);
      if (lookup_index(rel) != want) {
        if (bad_idx < 5) std::printf("index mismatch: rel %a got %d want %d\n", rel, lookup_index(rel), want);
        ++bad_idx;
      }
    }
    // 2. product: w is 1, a float in (0, 1], or a product of earlier table factors
    float w;
    switch (g() % 3) {
      case 0: w = 1.f; break;
      case 1: w = (float)U(g); break;
      default: w = (float)((double)lhi[1 + g() % 1000] * lut[1 + g() % 1000]); break;
    }
    const int k = (int)(g() % 1001);
    float y;
    if (!round_pair(ff_mul(FF{w, 0.f}, FF{lhi[k], llo[k]}), y)) continue;
    ++certified;
    const float want = (float)((double)w * lut[k]);
    if (bits_of(y) != bits_of(want)) {
      if (bad_prod < 5) std::printf("product mismatch: w %a k %d got %a want %a\n", w, k, y, want);
      ++bad_prod;
    }
  }
  std::printf("index %lld mismatches %lld product %lld certified %lld mismatches %lld\n", cases, bad_idx, cases,
              certified, bad_prod);
  return (bad_idx || bad_prod) ? 1 : 0;
}
