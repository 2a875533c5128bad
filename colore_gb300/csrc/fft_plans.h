/*
 * fft_plans.h -- per-grid-size plans of the 3-D c2r transform: radices and
 * elements per thread of the length-N column transforms of the y pass (CR,
 * C0-C2) and of the fused fill + z pass (FR, F0-F2: fewer elements per
 * thread, so that more threads share the mode generation), of the
 * length-N/2 row transforms of the x pass (RR, R0-R2), tile widths of the
 * column passes (TX2: fill with two fields, TX3: fill with three fields, TXY:
 * y pass) and rows per block of the x pass.
 */
#ifndef CG_FFT_PLANS_H
#define CG_FFT_PLANS_H

namespace {

template <int N>
struct Plan;
#define CG_PLAN(N_, CR_, C0_, C1_, C2_, FR_, F0_, F1_, F2_, TX2_, TX3_, TXY_, RR_, R0_, R1_, R2_, RB_) \
  template <>                                                                                     \
  struct Plan<N_> {                                                                               \
    static constexpr int CR = CR_, C0 = C0_, C1 = C1_, C2 = C2_;                                  \
    static constexpr int FR = FR_, F0 = F0_, F1 = F1_, F2 = F2_;                                  \
    static constexpr int TX2 = TX2_, TX3 = TX3_, TXY = TXY_;                                      \
    static constexpr int RR = RR_, R0 = R0_, R1 = R1_, R2 = R2_, RB = RB_;                        \
  };
/*      N    CR  C0  C1 C2  FR  F0  F1 F2 TX2 TX3 TXY  RR  R0  R1 R2 RB */
CG_PLAN(64, 8, 8, 8, 1, 8, 8, 8, 1, 32, 16, 32, 8, 8, 4, 1, 16)
CG_PLAN(96, 24, 24, 4, 1, 12, 12, 4, 2, 32, 16, 32, 12, 12, 4, 1, 16)
CG_PLAN(128, 16, 16, 8, 1, 8, 8, 8, 2, 32, 16, 32, 8, 8, 8, 1, 16)
CG_PLAN(192, 24, 24, 8, 1, 12, 12, 4, 4, 16, 16, 32, 24, 24, 4, 1, 16)
CG_PLAN(256, 16, 16, 16, 1, 16, 16, 16, 1, 16, 16, 32, 16, 16, 8, 1, 16)
CG_PLAN(384, 24, 24, 4, 4, 24, 24, 4, 4, 16, 8, 16, 24, 24, 8, 1, 16)
CG_PLAN(512, 32, 32, 16, 1, 16, 16, 16, 2, 8, 8, 8, 16, 16, 16, 1, 8)
CG_PLAN(1024, 32, 32, 32, 1, 16, 16, 16, 4, 4, 4, 8, 32, 32, 16, 1, 8)
CG_PLAN(2048, 32, 32, 32, 2, 16, 16, 16, 8, 4, 2, 8, 32, 32, 32, 1, 4)
#undef CG_PLAN

} /* namespace */

#endif
