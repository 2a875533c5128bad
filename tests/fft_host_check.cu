// Host check of the transform building blocks of colore_gb300/csrc/fft.cuh:
// emulates cgfft::transform stage by stage (the same DFT kernels, twiddles
// and Stockham positions, evaluated on the CPU in float) for every plan of
// fft_plans.h, and prints the max error against an FP64 DFT per length.
#include <cmath>
#include <complex>
#include <cstdio>
#include <vector>

#include "fft.cuh"
#include "fft_plans.h"

using cplx = std::complex<double>;

template <int L, int R, int r0, int r1, int r2>
static double check_plan(unsigned seed)
{
  constexpr int P = L / R;
  std::vector<float2> x(L), tw(L), buf(L), v((size_t)P * R), y(L);
  for (int j = 0; j < L; j++) tw[j] = make_float2((float)cos(2 * M_PI * j / L), (float)sin(2 * M_PI * j / L));
  unsigned s = seed;
  for (int j = 0; j < L; j++) {
    s = s * 1664525u + 1013904223u;
    float a = (float)((s >> 8) & 0xffff) / 65536.0f - 0.5f;
    s = s * 1664525u + 1013904223u;
    float b = (float)((s >> 8) & 0xffff) / 65536.0f - 0.5f;
    x[j] = make_float2(a, b);
  }
  auto run_stage = [&](auto rc, auto nsc, bool first) {
    constexpr int r = decltype(rc)::value, Ns = decltype(nsc)::value;
    for (int t = 0; t < P; t++) {
      float2 *vt = &v[(size_t)t * R];
      for (int i = 0; i < R / r; i++)
        for (int q = 0; q < r; q++)
          vt[i * r + q] = first ? x[cgfft::in_pos<L, R, r>(t, i, q)] : buf[cgfft::in_pos<L, R, r>(t, i, q)];
      cgfft::stage<L, R, r, Ns, 1>(vt, t, tw.data());
    }
    std::vector<float2> out(L);
    for (int t = 0; t < P; t++)
      for (int i = 0; i < R / r; i++)
        for (int q = 0; q < r; q++) out[cgfft::out_pos<L, R, r, Ns>(t, i, q)] = v[(size_t)t * R + i * r + q];
    buf = out;
  };
  run_stage(std::integral_constant<int, r0>(), std::integral_constant<int, 1>(), true);
  if (r1 > 1) run_stage(std::integral_constant<int, (r1 > 1 ? r1 : 2)>(), std::integral_constant<int, r0>(), false);
  if (r2 > 1)
    run_stage(std::integral_constant<int, (r2 > 1 ? r2 : 2)>(), std::integral_constant<int, r0 * (r1 > 1 ? r1 : 1)>(),
              false);
  double err = 0, nrm = 0;
  for (int k = 0; k < L; k++) {
    cplx acc = 0;
    for (int n = 0; n < L; n++) acc += cplx(x[n].x, x[n].y) * std::polar(1.0, 2 * M_PI * (double)((long)k * n % L) / L);
    err = std::fmax(err, std::abs(acc - cplx(buf[k].x, buf[k].y)));
    nrm = std::fmax(nrm, std::abs(acc));
  }
  return err / nrm;
}

template <int N>
static void check_size()
{
  using PL = Plan<N>;
  double ec = check_plan<N, PL::CR, PL::C0, PL::C1, PL::C2>(N);
  double ef = check_plan<N, PL::FR, PL::F0, PL::F1, PL::F2>(N + 2);
  double er = check_plan<N / 2, PL::RR, PL::R0, PL::R1, PL::R2>(N + 1);
  printf("%d %.3e %.3e\n", N, ec > ef ? ec : ef, er);
}

int main()
{
  check_size<64>();
  check_size<96>();
  check_size<128>();
  check_size<192>();
  check_size<256>();
  check_size<384>();
  check_size<512>();
  check_size<1024>();
  check_size<2048>();
  return 0;
}
