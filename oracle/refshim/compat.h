/*
 * compat.h -- force-included (-include) into every translation unit of the
 * Linux build of the reference pipeline core (oracle/_ref).  TEST
 * INFRASTRUCTURE ONLY: nothing in the product links or includes it.
 *
 * The reference (CallMeZhou/Puresoft3D) is MSVC/Win32 code.  This header maps
 * the handful of MSVC spellings it uses onto GCC/glibc equivalents with the
 * same meaning, so that the reference sources compile unmodified:
 *   __declspec(align(n))          -> nothing.  GCC cannot attach the
 *       alignment to an anonymous struct through a leading typedef attribute
 *       (reference proc.h:20-24 would become an array of under-sized
 *       over-aligned elements).  Alignment never changes a result: the
 *       stand-in maths library and the patched asm blocks use unaligned SSE
 *       loads/stores, and heap buffers still come from _aligned_malloc.
 *   __stdcall / _stdcall          -> nothing (x86-64 has one calling convention)
 *   _aligned_malloc/_aligned_free -> posix_memalign/free
 * Win32 threads and Interlocked* live in win32/windows.h + win32/process.h.
 */
#pragma once
#include <stdint.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <float.h>
#include <wchar.h>
#include <stdio.h>
#ifdef __cplusplus
#include <stdexcept> /* MSVC's <vector>/<stdlib.h> pull these in implicitly */
#include <new>
#endif

#define __declspec(x)
#define __stdcall
#define _stdcall

static inline void* _aligned_malloc(size_t bytes, size_t alignment)
{
    void* p = NULL;
    if (alignment < sizeof(void*)) alignment = sizeof(void*);
    if (posix_memalign(&p, alignment, bytes ? bytes : alignment) != 0) return NULL;
    return p;
}

static inline void _aligned_free(void* p) { free(p); }
