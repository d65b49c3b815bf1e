// Large-radix Stockham FFT building blocks for sm_103a (FP32).
//
// A transform of length N = R_0 R_1 ... R_{S-1} (each R_s <= 20, S usually 2) runs as S
// stages.  In stage s every butterfly reads R_s values (stride N / R_s), twiddles them, runs
// an R_s-point DFT in registers and writes them in Stockham (self-sorting) order.  Loads and
// stores go through functors, so the first stage can read straight from global memory, the
// last stage can write straight to global memory (or into an epilogue), and only the S - 1
// exchanges in between touch shared memory.  For a convolution the forward transform's last
// stage, the pointwise product with the kernel spectrum and the inverse transform's first
// stage (radix order reversed) run in the same registers, with no exchange at all.
//
// Butterfly b of `count` sequences maps to (batch, j) either batch-fastest (consecutive
// threads take consecutive sequences: column transforms and pencils, coalesced and free of
// bank conflicts) or j-fastest (consecutive threads take consecutive positions of one
// sequence: row transforms that load from or store to global memory).
//
// Twiddles between stages come from a per-length table exp(-2 pi i k / N) computed in double
// on the host; the internal roots of the composite register DFTs are compile-time tables
// (dft_consts.cuh).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "dft_consts.cuh"

namespace mvd {

constexpr int kMaxStages = 6;

// Runtime plan of one transform length (device copy lives in a plan table).
struct FftPlan {
  int n;                    // transform length
  int nstages;              // number of radix stages
  int radix[kMaxStages];    // radices (each in {2,3,4,5,6,8,9,10,12,15,16,18,20}), product == n
  const float2* tw;         // exp(-2 pi i k / n), k in [0, n)
  const float2* tw_r2c;     // for the real-input length 2n: exp(-2 pi i k / (2n)), k in [0, n]
};

__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
  return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
__device__ __forceinline__ float2 cconj(float2 a) { return make_float2(a.x, -a.y); }
// multiply by -i (forward) or +i (inverse)
template <bool INV>
__device__ __forceinline__ float2 mul_mi(float2 a) {
  return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

// ---------------------------------------------------------------------------------------
// R-point DFTs in registers.  Forward uses exp(-2 pi i / R); inverse the conjugate root.
// ---------------------------------------------------------------------------------------
template <int R, bool INV>
struct Dft;

template <bool INV>
struct Dft<1, INV> {
  __device__ __forceinline__ static void run(float2*) {}
};

template <bool INV>
struct Dft<2, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <bool INV>
struct Dft<4, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    float2 s0 = cadd(v[0], v[2]), d0 = csub(v[0], v[2]);
    float2 s1 = cadd(v[1], v[3]), d1 = mul_mi<INV>(csub(v[1], v[3]));
    v[0] = cadd(s0, s1);
    v[2] = csub(s0, s1);
    v[1] = cadd(d0, d1);
    v[3] = csub(d0, d1);
  }
};

template <bool INV>
struct Dft<8, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    const float h = 0.70710678118654752440f;  // sqrt(1/2)
    float2 e[4] = {v[0], v[2], v[4], v[6]};
    float2 o[4] = {v[1], v[3], v[5], v[7]};
    Dft<4, INV>::run(e);
    Dft<4, INV>::run(o);
    float2 o1 = o[1], o2 = o[2], o3 = o[3];
    o[1] = INV ? make_float2(h * (o1.x - o1.y), h * (o1.x + o1.y))
               : make_float2(h * (o1.x + o1.y), h * (o1.y - o1.x));
    o[2] = mul_mi<INV>(o2);
    o[3] = INV ? make_float2(-h * (o3.x + o3.y), h * (o3.x - o3.y))
               : make_float2(h * (o3.y - o3.x), -h * (o3.x + o3.y));
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      v[k] = cadd(e[k], o[k]);
      v[k + 4] = csub(e[k], o[k]);
    }
  }
};

template <bool INV>
struct Dft<3, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    const float c = -0.5f;
    const float s = 0.86602540378443864676f;  // sin(2 pi / 3)
    float2 a = cadd(v[1], v[2]);
    float2 b = csub(v[1], v[2]);
    float2 t = make_float2(v[0].x + c * a.x, v[0].y + c * a.y);
    float2 u = mul_mi<INV>(cscale(b, s));
    v[0] = cadd(v[0], a);
    v[1] = cadd(t, u);
    v[2] = csub(t, u);
  }
};

template <bool INV>
struct Dft<5, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    const float c1 = 0.30901699437494742410f;   // cos(2 pi / 5)
    const float c2 = -0.80901699437494742410f;  // cos(4 pi / 5)
    const float s1 = 0.95105651629515357212f;   // sin(2 pi / 5)
    const float s2 = 0.58778525229247312917f;   // sin(4 pi / 5)
    float2 p1 = cadd(v[1], v[4]), m1 = csub(v[1], v[4]);
    float2 p2 = cadd(v[2], v[3]), m2 = csub(v[2], v[3]);
    float2 x0 = v[0];
    float2 a1 = make_float2(x0.x + c1 * p1.x + c2 * p2.x, x0.y + c1 * p1.y + c2 * p2.y);
    float2 a2 = make_float2(x0.x + c2 * p1.x + c1 * p2.x, x0.y + c2 * p1.y + c1 * p2.y);
    float2 b1 = make_float2(s1 * m1.x + s2 * m2.x, s1 * m1.y + s2 * m2.y);
    float2 b2 = make_float2(s2 * m1.x - s1 * m2.x, s2 * m1.y - s1 * m2.y);
    float2 jb1 = mul_mi<INV>(b1), jb2 = mul_mi<INV>(b2);
    v[0] = make_float2(x0.x + p1.x + p2.x, x0.y + p1.y + p2.y);
    v[1] = cadd(a1, jb1);
    v[4] = csub(a1, jb1);
    v[2] = cadd(a2, jb2);
    v[3] = csub(a2, jb2);
  }
};

template <bool INV>
struct Dft<7, INV> {
  __device__ __forceinline__ static void run(float2* v) {
    // cos / sin of 2 pi k / 7, k = 1..3
    const float c[3] = {0.62348980185873353053f, -0.22252093395631440429f, -0.90096886790241912624f};
    const float s[3] = {0.78183148246802980871f, 0.97492791218182360702f, 0.43388373911755812048f};
    float2 p[3], m[3];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      p[k] = cadd(v[k + 1], v[6 - k]);
      m[k] = csub(v[k + 1], v[6 - k]);
    }
    float2 x0 = v[0];
    float2 out[7];
    out[0] = make_float2(x0.x + p[0].x + p[1].x + p[2].x, x0.y + p[0].y + p[1].y + p[2].y);
#pragma unroll
    for (int k = 1; k <= 3; ++k) {
      float2 a = x0, b = make_float2(0.f, 0.f);
#pragma unroll
      for (int n = 1; n <= 3; ++n) {
        const int idx = (k * n) % 7;  // cos(2 pi k n / 7) = c[min(idx, 7-idx) - 1]
        const int j = (idx <= 3 ? idx : 7 - idx) - 1;
        const float sg = idx <= 3 ? 1.f : -1.f;  // sign of sin(2 pi k n / 7)
        a.x += c[j] * p[n - 1].x;
        a.y += c[j] * p[n - 1].y;
        b.x += sg * s[j] * m[n - 1].x;
        b.y += sg * s[j] * m[n - 1].y;
      }
      float2 jb = mul_mi<INV>(b);
      out[k] = cadd(a, jb);
      out[7 - k] = csub(a, jb);
    }
#pragma unroll
    for (int k = 0; k < 7; ++k) v[k] = out[k];
  }
};

// R = A * B by one Cooley-Tukey split: n = B n1 + n2, k = k1 + A k2;
// X[k1 + A k2] = sum_n2 W_B^{n2 k2} W_R^{n2 k1} sum_n1 x[B n1 + n2] W_A^{n1 k1}
template <int A, int B, bool INV>
struct DftAB {
  __device__ __forceinline__ static void run(float2* v) {
    constexpr int R = A * B;
    float2 y[B][A];
#pragma unroll
    for (int n2 = 0; n2 < B; ++n2) {
      float2 t[A];
#pragma unroll
      for (int n1 = 0; n1 < A; ++n1) t[n1] = v[B * n1 + n2];
      Dft<A, INV>::run(t);
#pragma unroll
      for (int k1 = 0; k1 < A; ++k1) {
        if ((n2 * k1) % R == 0) {
          y[n2][k1] = t[k1];
        } else {
          float2 w = wconst<R>((n2 * k1) % R);
          if (INV) w.y = -w.y;
          y[n2][k1] = cmul(t[k1], w);
        }
      }
    }
#pragma unroll
    for (int k1 = 0; k1 < A; ++k1) {
      float2 t[B];
#pragma unroll
      for (int n2 = 0; n2 < B; ++n2) t[n2] = y[n2][k1];
      Dft<B, INV>::run(t);
#pragma unroll
      for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = t[k2];
    }
  }
};

template <bool INV> struct Dft<6, INV> : DftAB<2, 3, INV> {};
template <bool INV> struct Dft<9, INV> : DftAB<3, 3, INV> {};
template <bool INV> struct Dft<10, INV> : DftAB<2, 5, INV> {};
template <bool INV> struct Dft<12, INV> : DftAB<4, 3, INV> {};
template <bool INV> struct Dft<14, INV> : DftAB<2, 7, INV> {};
template <bool INV> struct Dft<15, INV> : DftAB<3, 5, INV> {};
template <bool INV> struct Dft<16, INV> : DftAB<4, 4, INV> {};
template <bool INV> struct Dft<18, INV> : DftAB<2, 9, INV> {};
template <bool INV> struct Dft<20, INV> : DftAB<4, 5, INV> {};

// ---------------------------------------------------------------------------------------
// butterfly index mapping
// ---------------------------------------------------------------------------------------
template <bool JFAST>
__device__ __forceinline__ void butterfly_index(int b, int count, int NR, int& batch, int& j) {
  if (JFAST) {
    batch = b / NR;
    j = b - batch * NR;
  } else {
    j = b / count;
    batch = b - j * count;
  }
}

// Whole-butterfly access: a functor may define get<R>(batch, j, NR, v) (v[r] = element
// j + r NR) and put<R>(batch, base, Ns, v) (element base + r Ns = v[r]) to batch its memory
// operations; these defaults use the per-element operators.
struct ElemAccess {
  template <int R, class F>
  __device__ __forceinline__ static void get(const F& f, int batch, int j, int NR, float2* v) {
#pragma unroll
    for (int r = 0; r < R; ++r) v[r] = f(batch, j + r * NR);
  }
  template <int R, class F>
  __device__ __forceinline__ static void put(const F& f, int batch, int base, int Ns, const float2* v) {
#pragma unroll
    for (int r = 0; r < R; ++r) f(batch, base + r * Ns, v[r]);
  }
};

// One radix-R Stockham stage of `count` sequences: ld.get<R>(...) and st.put<R>(...).
// Butterflies b = tid, tid + T, ... are walked with an incremental (batch, j) (no integer
// division in the loop) and k = j mod Ns is taken through an exact float reciprocal.
template <int R, bool INV, bool JFAST, class LD, class ST>
__device__ __forceinline__ void stage_r(int N, int Ns, int count, const float2* __restrict__ tw, const LD& ld,
                                        const ST& st) {
  const int NR = N / R;
  const int nb = count * NR;
  const int twstride = N / (Ns * R);
  const int T = blockDim.x;
  // fast and slow extents of the (batch, j) walk
  const int fast = JFAST ? NR : count;
  int f, sl;  // fast / slow coordinates of butterfly threadIdx.x
  {
    const int b = threadIdx.x;
    sl = b / fast;
    f = b - sl * fast;
  }
  const int dsl = T / fast, df = T - dsl * fast;
  const float inv_ns = 1.0f / (float)Ns;
  for (int b = threadIdx.x; b < nb; b += T) {
    const int batch = JFAST ? sl : f;
    const int j = JFAST ? f : sl;
    float2 v[R];
    ld.template get<R>(batch, j, NR, v);
    int k = 0;
    if (Ns > 1) {
      k = j - Ns * (int)((float)j * inv_ns);  // exact for j < 2^22 up to one step
      if (k < 0) k += Ns;
      if (k >= Ns) k -= Ns;
    }
    if (k != 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) {
        float2 w = __ldg(tw + r * k * twstride);
        if (INV) w.y = -w.y;
        v[r] = cmul(v[r], w);
      }
    }
    Dft<R, INV>::run(v);
    st.template put<R>(batch, (j - k) * R + k, Ns, v);
    f += df;
    sl += dsl;
    if (f >= fast) {
      f -= fast;
      sl += 1;
    }
  }
}

template <bool INV, bool JFAST, class LD, class ST>
__device__ __forceinline__ void stage(int R, int N, int Ns, int count, const float2* __restrict__ tw, const LD& ld,
                                      const ST& st) {
  switch (R) {
    case 2: stage_r<2, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 3: stage_r<3, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 4: stage_r<4, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 5: stage_r<5, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 6: stage_r<6, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 8: stage_r<8, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 9: stage_r<9, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 10: stage_r<10, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 12: stage_r<12, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 15: stage_r<15, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 16: stage_r<16, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 18: stage_r<18, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    case 20: stage_r<20, INV, JFAST>(N, Ns, count, tw, ld, st); break;
    default: stage_r<1, INV, JFAST>(N, Ns, count, tw, ld, st); break;  // length-1 transform: copy
  }
}

// Forward last stage (radix R, Ns = N/R) + pointwise product + inverse first stage (radix R,
// Ns = 1) in the same registers.  mul(batch, k, v) returns v times the spectrum at natural
// index k.  Output: the inverse first stage's Stockham order (index j R + r).
template <int R, class LD, class MUL, class ST>
__device__ __forceinline__ void zmid_r(int N, int count, const float2* __restrict__ tw, const LD& ld, const MUL& mul,
                                       const ST& st) {
  const int NR = N / R;
  const int nb = count * NR;
  for (int b = threadIdx.x; b < nb; b += blockDim.x) {
    int batch, j;
    butterfly_index<false>(b, count, NR, batch, j);
    float2 v[R];
    ld.template get<R>(batch, j, NR, v);
    if (j != 0) {
#pragma unroll
      for (int r = 1; r < R; ++r) v[r] = cmul(v[r], __ldg(tw + r * j));
    }
    Dft<R, false>::run(v);
    mul.template apply<R>(batch, j, NR, v);
    Dft<R, true>::run(v);
    st.template put<R>(batch, j * R, 1, v);
  }
}

template <class LD, class MUL, class ST>
__device__ __forceinline__ void zmid(int R, int N, int count, const float2* __restrict__ tw, const LD& ld,
                                     const MUL& mul, const ST& st) {
  switch (R) {
    case 2: zmid_r<2>(N, count, tw, ld, mul, st); break;
    case 3: zmid_r<3>(N, count, tw, ld, mul, st); break;
    case 4: zmid_r<4>(N, count, tw, ld, mul, st); break;
    case 5: zmid_r<5>(N, count, tw, ld, mul, st); break;
    case 6: zmid_r<6>(N, count, tw, ld, mul, st); break;
    case 8: zmid_r<8>(N, count, tw, ld, mul, st); break;
    case 9: zmid_r<9>(N, count, tw, ld, mul, st); break;
    case 10: zmid_r<10>(N, count, tw, ld, mul, st); break;
    case 12: zmid_r<12>(N, count, tw, ld, mul, st); break;
    case 15: zmid_r<15>(N, count, tw, ld, mul, st); break;
    case 16: zmid_r<16>(N, count, tw, ld, mul, st); break;
    case 18: zmid_r<18>(N, count, tw, ld, mul, st); break;
    case 20: zmid_r<20>(N, count, tw, ld, mul, st); break;
    default: zmid_r<1>(N, count, tw, ld, mul, st); break;
  }
}

// ---------------------------------------------------------------------------------------
// Shared-memory accessor: element (batch, i) at p[batch * bs + s(i) * es], where s(i) = i, or
// i + i/16 for the skewed row layout (one type for every exchange keeps the code small).
// ---------------------------------------------------------------------------------------
struct Smem {
  float2* p;
  int es, bs, skew;
  __device__ __forceinline__ int at(int batch, int i) const { return batch * bs + (i + ((i >> 4) & skew)) * es; }
  __device__ __forceinline__ float2 operator()(int batch, int i) const { return p[at(batch, i)]; }
  __device__ __forceinline__ void operator()(int batch, int i, float2 v) const { p[at(batch, i)] = v; }
  template <int R>
  __device__ __forceinline__ void get(int batch, int j, int NR, float2* v) const {
    if (skew) {
      ElemAccess::get<R>(*this, batch, j, NR, v);
    } else {  // base pointer and constant stride
      const float2* q = p + batch * bs + j * es;
      const int st = NR * es;
#pragma unroll
      for (int r = 0; r < R; ++r) v[r] = q[r * st];
    }
  }
  template <int R>
  __device__ __forceinline__ void put(int batch, int base, int Ns, const float2* v) const {
    if (skew) {
      ElemAccess::put<R>(*this, batch, base, Ns, v);
    } else {
      float2* q = p + batch * bs + base * es;
      const int st = Ns * es;
#pragma unroll
      for (int r = 0; r < R; ++r) q[r * st] = v[r];
    }
  }
};

}  // namespace mvd
