// Forced-include header of the reference harness's contact-margin variant (test infrastructure
// only; oracle/build_ref.py passes it with -include and -DPE_MARGIN_VALUE=...).
//
// The reference fixes its contact margin at compile time: PE_MARGIN is pe::Real(0)
// (src/rigid/phys_general.h:45), and every collision algorithm reads it into a constexpr.  This
// header includes phys_general.h first (its #pragma once keeps it from being read again) and
// then redefines the constant, so the reference's own sources compile unchanged with another
// margin.
#pragma once
#include "rigid/phys_general.h"
#undef PE_MARGIN
#define PE_MARGIN pe::Real(PE_MARGIN_VALUE)
