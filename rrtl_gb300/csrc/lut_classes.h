// The 80 LUT3 truth tables that represent their class under input
// permutation (each is the smallest table among the six input orders of its
// function; the gate lowering reorders every cell's inputs to reach it, see
// canonicalize_inputs). The fused kernel specialises one loop per entry; a
// per-design compiled fused kernel defines RRTL_LUT_CLASSES first with only
// the classes its design uses (and 0, the class of an empty run).
#pragma once

#ifndef RRTL_LUT_CLASSES
#define RRTL_LUT_CLASSES(X) \
  X(0) X(1) X(2) X(3) X(6) X(7) X(8) X(9) X(10) X(11) \
  X(14) X(15) X(22) X(23) X(24) X(25) X(26) X(27) X(30) X(31) \
  X(40) X(41) X(42) X(43) X(44) X(45) X(46) X(47) X(60) X(61) \
  X(62) X(63) X(104) X(105) X(106) X(107) X(110) X(111) X(126) X(127) \
  X(128) X(129) X(130) X(131) X(134) X(135) X(136) X(137) X(138) X(139) \
  X(142) X(143) X(150) X(151) X(152) X(153) X(154) X(155) X(158) X(159) \
  X(168) X(169) X(170) X(171) X(172) X(173) X(174) X(175) X(188) X(189) \
  X(190) X(191) X(232) X(233) X(234) X(235) X(238) X(239) X(254) X(255)
#endif
