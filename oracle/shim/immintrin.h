/*
 * Empty stand-in for <immintrin.h> on non-x86 hosts (test infrastructure).
 *
 * The reference's decoder dispatch file includes its AVX2 / AVX-512 headers
 * unconditionally, and those include <immintrin.h>, although with
 * ARCH_X86_64 undefined nothing of the x86 intrinsics is used: the headers
 * are needed only for prototypes that use plain C types.  oracle/Makefile puts
 * this directory first on the include path on such hosts so that the
 * reference's portable C path builds there as the CPU baseline.
 */
#ifndef JXS_SHIM_IMMINTRIN_H
#define JXS_SHIM_IMMINTRIN_H
#endif
