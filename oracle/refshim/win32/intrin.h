/* intrin.h stand-in (oracle/_ref, TEST INFRASTRUCTURE ONLY): the reference's
   fbo.cpp uses MMX/SSE intrinsics (blend4, blend16); GCC declares them here. */
#pragma once
#include <x86intrin.h>
