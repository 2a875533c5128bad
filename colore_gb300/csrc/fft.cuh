/*
 * fft.cuh -- building blocks of the FP32 3-D c2r transform on sm_103a.
 *
 * A length-L complex transform is split into Stockham stages of radix r
 * (L = r0 r1 r2).  Each of the P = L/R threads of a transform holds R
 * elements in registers; a stage applies the inter-stage twiddles and R/r
 * radix-r DFTs in registers, and consecutive stages exchange data through
 * shared memory once.  Stage 0 takes its inputs from a loader functor (a
 * global read, a generator, or a shared-memory staging buffer) and the last
 * stage hands its outputs to a storer functor, so loads and stores go
 * straight between HBM and registers.
 *
 * Stage s with radix r and span Ns (product of the previous radices), for
 * butterfly b in [0, L/r):
 *   inputs  x[b + q L/r],                     q = 0..r-1
 *   twiddle x_q *= exp(S 2 pi i q (b mod Ns) / (Ns r))
 *   outputs y[(b div Ns) Ns r + (b mod Ns) + q Ns] = DFT_r(x)_q
 * (Stockham autosort; output in natural order, no bit reversal).
 */
#ifndef CG_FFT_CUH
#define CG_FFT_CUH

#include <cuda_runtime.h>

namespace cgfft {

/* exp(+2 pi i j / 96), j = 0..95: every radix used here divides 96. */
#define CG_TW96_VALUES \
  { \
    {1.000000000e+00f, 0.000000000e+00f}, {9.978589416e-01f, 6.540312618e-02f}, \
    {9.914448857e-01f, 1.305261850e-01f}, {9.807852507e-01f, 1.950903237e-01f}, \
    {9.659258127e-01f, 2.588190436e-01f}, {9.469301105e-01f, 3.214394748e-01f}, \
    {9.238795042e-01f, 3.826834261e-01f}, {8.968727589e-01f, 4.422886968e-01f}, \
    {8.660253882e-01f, 5.000000000e-01f}, {8.314695954e-01f, 5.555702448e-01f}, \
    {7.933533192e-01f, 6.087614298e-01f}, {7.518398166e-01f, 6.593458056e-01f}, \
    {7.071067691e-01f, 7.071067691e-01f}, {6.593458056e-01f, 7.518398166e-01f}, \
    {6.087614298e-01f, 7.933533192e-01f}, {5.555702448e-01f, 8.314695954e-01f}, \
    {5.000000000e-01f, 8.660253882e-01f}, {4.422886968e-01f, 8.968727589e-01f}, \
    {3.826834261e-01f, 9.238795042e-01f}, {3.214394748e-01f, 9.469301105e-01f}, \
    {2.588190436e-01f, 9.659258127e-01f}, {1.950903237e-01f, 9.807852507e-01f}, \
    {1.305261850e-01f, 9.914448857e-01f}, {6.540312618e-02f, 9.978589416e-01f}, \
    {0.000000000e+00f, 1.000000000e+00f}, {-6.540312618e-02f, 9.978589416e-01f}, \
    {-1.305261850e-01f, 9.914448857e-01f}, {-1.950903237e-01f, 9.807852507e-01f}, \
    {-2.588190436e-01f, 9.659258127e-01f}, {-3.214394748e-01f, 9.469301105e-01f}, \
    {-3.826834261e-01f, 9.238795042e-01f}, {-4.422886968e-01f, 8.968727589e-01f}, \
    {-5.000000000e-01f, 8.660253882e-01f}, {-5.555702448e-01f, 8.314695954e-01f}, \
    {-6.087614298e-01f, 7.933533192e-01f}, {-6.593458056e-01f, 7.518398166e-01f}, \
    {-7.071067691e-01f, 7.071067691e-01f}, {-7.518398166e-01f, 6.593458056e-01f}, \
    {-7.933533192e-01f, 6.087614298e-01f}, {-8.314695954e-01f, 5.555702448e-01f}, \
    {-8.660253882e-01f, 5.000000000e-01f}, {-8.968727589e-01f, 4.422886968e-01f}, \
    {-9.238795042e-01f, 3.826834261e-01f}, {-9.469301105e-01f, 3.214394748e-01f}, \
    {-9.659258127e-01f, 2.588190436e-01f}, {-9.807852507e-01f, 1.950903237e-01f}, \
    {-9.914448857e-01f, 1.305261850e-01f}, {-9.978589416e-01f, 6.540312618e-02f}, \
    {-1.000000000e+00f, 0.000000000e+00f}, {-9.978589416e-01f, -6.540312618e-02f}, \
    {-9.914448857e-01f, -1.305261850e-01f}, {-9.807852507e-01f, -1.950903237e-01f}, \
    {-9.659258127e-01f, -2.588190436e-01f}, {-9.469301105e-01f, -3.214394748e-01f}, \
    {-9.238795042e-01f, -3.826834261e-01f}, {-8.968727589e-01f, -4.422886968e-01f}, \
    {-8.660253882e-01f, -5.000000000e-01f}, {-8.314695954e-01f, -5.555702448e-01f}, \
    {-7.933533192e-01f, -6.087614298e-01f}, {-7.518398166e-01f, -6.593458056e-01f}, \
    {-7.071067691e-01f, -7.071067691e-01f}, {-6.593458056e-01f, -7.518398166e-01f}, \
    {-6.087614298e-01f, -7.933533192e-01f}, {-5.555702448e-01f, -8.314695954e-01f}, \
    {-5.000000000e-01f, -8.660253882e-01f}, {-4.422886968e-01f, -8.968727589e-01f}, \
    {-3.826834261e-01f, -9.238795042e-01f}, {-3.214394748e-01f, -9.469301105e-01f}, \
    {-2.588190436e-01f, -9.659258127e-01f}, {-1.950903237e-01f, -9.807852507e-01f}, \
    {-1.305261850e-01f, -9.914448857e-01f}, {-6.540312618e-02f, -9.978589416e-01f}, \
    {0.000000000e+00f, -1.000000000e+00f}, {6.540312618e-02f, -9.978589416e-01f}, \
    {1.305261850e-01f, -9.914448857e-01f}, {1.950903237e-01f, -9.807852507e-01f}, \
    {2.588190436e-01f, -9.659258127e-01f}, {3.214394748e-01f, -9.469301105e-01f}, \
    {3.826834261e-01f, -9.238795042e-01f}, {4.422886968e-01f, -8.968727589e-01f}, \
    {5.000000000e-01f, -8.660253882e-01f}, {5.555702448e-01f, -8.314695954e-01f}, \
    {6.087614298e-01f, -7.933533192e-01f}, {6.593458056e-01f, -7.518398166e-01f}, \
    {7.071067691e-01f, -7.071067691e-01f}, {7.518398166e-01f, -6.593458056e-01f}, \
    {7.933533192e-01f, -6.087614298e-01f}, {8.314695954e-01f, -5.555702448e-01f}, \
    {8.660253882e-01f, -5.000000000e-01f}, {8.968727589e-01f, -4.422886968e-01f}, \
    {9.238795042e-01f, -3.826834261e-01f}, {9.469301105e-01f, -3.214394748e-01f}, \
    {9.659258127e-01f, -2.588190436e-01f}, {9.807852507e-01f, -1.950903237e-01f}, \
    {9.914448857e-01f, -1.305261850e-01f}, {9.978589416e-01f, -6.540312618e-02f} \
  }
static __constant__ float2 c_tw96[96] = CG_TW96_VALUES;
static const float2 h_tw96[96] = CG_TW96_VALUES;
#ifdef __CUDA_ARCH__
#define CG_TW96(j) c_tw96[j]
#define CG_LDG(p) __ldg(p)
#else
#define CG_TW96(j) h_tw96[j]
#define CG_LDG(p) (*(p))
#endif

__host__ __device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__host__ __device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
__host__ __device__ __forceinline__ float2 cscale(float2 a, float s) { return make_float2(a.x * s, a.y * s); }
/* a * w (S>0) or a * conj(w) (S<0) */
template <int S>
__host__ __device__ __forceinline__ float2 cmulS(float2 a, float2 w)
{
  if (S > 0) return make_float2(a.x * w.x - a.y * w.y, a.x * w.y + a.y * w.x);
  return make_float2(a.x * w.x + a.y * w.y, a.y * w.x - a.x * w.y);
}
/* S * i * a */
template <int S>
__host__ __device__ __forceinline__ float2 mulSi(float2 a)
{
  return S > 0 ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
}

/* a * exp(S 2 pi i m / R) for a compile-time m once loops are unrolled */
template <int R, int S>
__host__ __device__ __forceinline__ float2 twc(float2 a, int m)
{
  int j = (m * (96 / R)) % 96;
  if (j == 0) return a;
  if (j == 24) return mulSi<S>(a);
  if (j == 48) return make_float2(-a.x, -a.y);
  if (j == 72) return mulSi<-S>(a);
  return cmulS<S>(a, CG_TW96(j));
}

template <int R, int S>
struct DFT;

template <int S>
struct DFT<2, S> {
  __host__ __device__ __forceinline__ static void run(float2 *v)
  {
    float2 a = v[0], b = v[1];
    v[0] = cadd(a, b);
    v[1] = csub(a, b);
  }
};

template <int S>
struct DFT<3, S> {
  __host__ __device__ __forceinline__ static void run(float2 *v)
  {
    const float s3 = 0.866025403784438647f;
    float2 a = v[0], b = v[1], c = v[2];
    float2 t1 = cadd(b, c);
    float2 t2 = make_float2(a.x - 0.5f * t1.x, a.y - 0.5f * t1.y);
    float2 t3 = mulSi<S>(cscale(csub(b, c), s3));
    v[0] = cadd(a, t1);
    v[1] = cadd(t2, t3);
    v[2] = csub(t2, t3);
  }
};

template <int S>
struct DFT<4, S> {
  __host__ __device__ __forceinline__ static void run(float2 *v)
  {
    float2 a = v[0], b = v[1], c = v[2], d = v[3];
    float2 s0 = cadd(a, c), s1 = csub(a, c), s2 = cadd(b, d), s3 = mulSi<S>(csub(b, d));
    v[0] = cadd(s0, s2);
    v[2] = csub(s0, s2);
    v[1] = cadd(s1, s3);
    v[3] = csub(s1, s3);
  }
};

/* Composite radix R = R1 R2 by one Cooley-Tukey split in registers. */
template <int R1, int R2, int S>
__host__ __device__ __forceinline__ void dft_split(float2 *v)
{
  constexpr int R = R1 * R2;
  float2 t[R];
#pragma unroll
  for (int n2 = 0; n2 < R2; n2++) {
    float2 a[R1];
#pragma unroll
    for (int n1 = 0; n1 < R1; n1++) a[n1] = v[R2 * n1 + n2];
    DFT<R1, S>::run(a);
#pragma unroll
    for (int k1 = 0; k1 < R1; k1++) t[n2 * R1 + k1] = twc<R, S>(a[k1], n2 * k1);
  }
#pragma unroll
  for (int k1 = 0; k1 < R1; k1++) {
    float2 b[R2];
#pragma unroll
    for (int n2 = 0; n2 < R2; n2++) b[n2] = t[n2 * R1 + k1];
    DFT<R2, S>::run(b);
#pragma unroll
    for (int k2 = 0; k2 < R2; k2++) v[k1 + R1 * k2] = b[k2];
  }
}

#define CG_DFT_SPLIT(R, R1, R2)                                            \
  template <int S>                                                         \
  struct DFT<R, S> {                                                       \
    __host__ __device__ __forceinline__ static void run(float2 *v) { dft_split<R1, R2, S>(v); } \
  };
CG_DFT_SPLIT(6, 3, 2)
CG_DFT_SPLIT(8, 4, 2)
CG_DFT_SPLIT(12, 4, 3)
CG_DFT_SPLIT(16, 4, 4)
CG_DFT_SPLIT(24, 8, 3)
CG_DFT_SPLIT(32, 8, 4)
CG_DFT_SPLIT(48, 16, 3)
CG_DFT_SPLIT(64, 8, 8)
#undef CG_DFT_SPLIT

/* Position read by stage input (i, q) of thread t. */
template <int L, int R, int r>
__host__ __device__ __forceinline__ int in_pos(int t, int i, int q)
{
  return t + (L / R) * i + q * (L / r);
}
/* Position written by stage output (i, q) of thread t. */
template <int L, int R, int r, int Ns>
__host__ __device__ __forceinline__ int out_pos(int t, int i, int q)
{
  int b = t + (L / R) * i;
  return (b / Ns) * Ns * r + (b % Ns) + q * Ns;
}

/* Twiddles and radix-r butterflies of one stage, data in v[i*r + q]. */
template <int L, int R, int r, int Ns, int S>
__host__ __device__ __forceinline__ void stage(float2 *v, int t, const float2 *__restrict__ twL)
{
  constexpr int NB = R / r;
#pragma unroll
  for (int i = 0; i < NB; i++) {
    if (Ns > 1) {
      int b = t + (L / R) * i;
      int k = b % Ns;
#pragma unroll
      for (int q = 1; q < r; q++) {
        float2 w = CG_LDG(&twL[(q * k) * (L / (Ns * r))]);
        v[i * r + q] = cmulS<S>(v[i * r + q], w);
      }
    }
    DFT<r, S>::run(&v[i * r]);
  }
}

/*
 * Full transform of length L = r0*r1*r2 (r2 = 1 for two stages, r1 = r2 = 1
 * for one) by P = L/R threads.  Ld(pos) -> float2 supplies the input,
 * St(pos, value) consumes the output, Sm(pos) -> float2& addresses this
 * transform's shared-memory exchange slot.  Contains the barriers of the
 * exchanges, so every thread of the block must call it.
 */
template <int L, int R, int r0, int r1, int r2, int S, class Ld, class St, class Sm>
__device__ __forceinline__ void transform(int t, const float2 *__restrict__ twL, Ld ld, St st, Sm sm)
{
  float2 v[R];
#pragma unroll
  for (int i = 0; i < R / r0; i++)
#pragma unroll
    for (int q = 0; q < r0; q++) v[i * r0 + q] = ld(in_pos<L, R, r0>(t, i, q));
  stage<L, R, r0, 1, S>(v, t, twL);
  if (r1 == 1) {
#pragma unroll
    for (int i = 0; i < R / r0; i++)
#pragma unroll
      for (int q = 0; q < r0; q++) st(out_pos<L, R, r0, 1>(t, i, q), v[i * r0 + q]);
    return;
  }
  constexpr int r1c = r1 > 1 ? r1 : 2; /* keeps templates valid when r1 == 1 */
  __syncthreads();
#pragma unroll
  for (int i = 0; i < R / r0; i++)
#pragma unroll
    for (int q = 0; q < r0; q++) sm(out_pos<L, R, r0, 1>(t, i, q)) = v[i * r0 + q];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < R / r1c; i++)
#pragma unroll
    for (int q = 0; q < r1c; q++) v[i * r1c + q] = sm(in_pos<L, R, r1c>(t, i, q));
  stage<L, R, r1c, r0, S>(v, t, twL);
  if (r2 == 1) {
#pragma unroll
    for (int i = 0; i < R / r1c; i++)
#pragma unroll
      for (int q = 0; q < r1c; q++) st(out_pos<L, R, r1c, r0>(t, i, q), v[i * r1c + q]);
    return;
  }
  constexpr int r2c = r2 > 1 ? r2 : 2;
  __syncthreads();
#pragma unroll
  for (int i = 0; i < R / r1c; i++)
#pragma unroll
    for (int q = 0; q < r1c; q++) sm(out_pos<L, R, r1c, r0>(t, i, q)) = v[i * r1c + q];
  __syncthreads();
#pragma unroll
  for (int i = 0; i < R / r2c; i++)
#pragma unroll
    for (int q = 0; q < r2c; q++) v[i * r2c + q] = sm(in_pos<L, R, r2c>(t, i, q));
  stage<L, R, r2c, r0 * r1c, S>(v, t, twL);
#pragma unroll
  for (int i = 0; i < R / r2c; i++)
#pragma unroll
    for (int q = 0; q < r2c; q++) st(out_pos<L, R, r2c, r0 * r1c>(t, i, q), v[i * r2c + q]);
}

} /* namespace cgfft */

#endif /* CG_FFT_CUH */
