// The reference's DE operators (cuda/src/semblance/kernel/common/
// differential_evolution.cu) compiled with F = 0.5 and CR = 0.9, the values
// of the DE workloads; the reference compiles F_FAC = 0.85 and CR = 0.5
// (common/include/gpu/interface.h:5-6).  interface.h is #pragma once, so the
// redefinitions below stand when the operator source includes it again.
// Test infrastructure: built by oracle/build_ref.py against the reference
// tree into oracle/_ref/.
#include "common/include/gpu/interface.h"
#undef F_FAC
#undef CR
#define F_FAC 0.5f
#define CR 0.9f
#include "cuda/src/semblance/kernel/common/differential_evolution.cu"
