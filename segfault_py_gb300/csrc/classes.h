// classes.h -- the 21 canonical shell-quartet classes (la lb | lc ld) with
// l <= 2 and the thread-group size T used for each.  T = 1 keeps the quartet
// in registers; FP32 needs half the registers of FP64, so classes up to 81
// Cartesian outputs stay register-resident in FP32.  Class id = X(X+1)/2 + Y
// for pair classes X >= Y (ss=0 ps=1 pp=2 ds=3 dp=4 dd=5).
//   X(id, la, lb, lc, ld, T_fp64, T_fp32)
#pragma once
#define SF_CLASS_LIST(X)       \
  X(0, 0, 0, 0, 0, 1, 1)       \
  X(1, 1, 0, 0, 0, 1, 1)       \
  X(2, 1, 0, 1, 0, 1, 1)       \
  X(3, 1, 1, 0, 0, 1, 1)       \
  X(4, 1, 1, 1, 0, 1, 1)       \
  X(5, 1, 1, 1, 1, 4, 1)       \
  X(6, 2, 0, 0, 0, 1, 1)       \
  X(7, 2, 0, 1, 0, 1, 1)       \
  X(8, 2, 0, 1, 1, 2, 1)       \
  X(9, 2, 0, 2, 0, 2, 1)       \
  X(10, 2, 1, 0, 0, 1, 1)      \
  X(11, 2, 1, 1, 0, 2, 1)      \
  X(12, 2, 1, 1, 1, 8, 8)      \
  X(13, 2, 1, 2, 0, 4, 4)      \
  X(14, 2, 1, 2, 1, 16, 16)    \
  X(15, 2, 2, 0, 0, 2, 1)      \
  X(16, 2, 2, 1, 0, 4, 4)      \
  X(17, 2, 2, 1, 1, 16, 16)    \
  X(18, 2, 2, 2, 0, 8, 8)      \
  X(19, 2, 2, 2, 1, 32, 32)    \
  X(20, 2, 2, 2, 2, 32, 32)

namespace sf {
struct ClassInfo { int la, lb, lc, ld, t64, t32; };
// Lanes per quartet of the double-float kernels run as the accurate tier of a
// mixed build: twice the FP64 lanes for classes with 18 or more outputs.
// That tier holds few quartets with long primitive loops (Q_ab Q_cd above
// the FP32 cutoff) and its launches are latency-bound, so fewer outputs and
// registers per lane and more warps shorten them ((H2O)8 6-31G* FP32 +
// double-float build 1.60 -> 1.39 ms); with every quartet in double-float the
// FP64 lanes stay better ((H2O)16: 24.2 ms against 25.5 ms).
constexpr int tdd_wide(int la, int lb, int lc, int ld, int t64) {
  return (la + 1) * (la + 2) / 2 * ((lb + 1) * (lb + 2) / 2) * ((lc + 1) * (lc + 2) / 2) * ((ld + 1) * (ld + 2) / 2) >= 18
             ? (2 * t64 < 32 ? 2 * t64 : 32)
             : t64;
}
constexpr ClassInfo kClassInfo[21] = {
#define SF_CI(id, la, lb, lc, ld, t64, t32) {la, lb, lc, ld, t64, t32},
    SF_CLASS_LIST(SF_CI)
#undef SF_CI
};
}  // namespace sf
