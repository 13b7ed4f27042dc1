/* Stand-in for the x86 intrinsics header.  The reference's helpers_CPU/
 * dynamicsGradient.h:16 includes <immintrin.h> but calls no intrinsic, so an
 * empty header lets oracle/_ref build from the reference's sources on any
 * host architecture (the Grace hosts of GB300 included). */
#pragma once
