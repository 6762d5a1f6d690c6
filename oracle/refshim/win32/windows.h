/*
 * windows.h stand-in for the Linux build of the reference pipeline core
 * (oracle/_ref).  TEST INFRASTRUCTURE ONLY.
 *
 * Provides exactly the Win32 surface the reference's pipeline core touches:
 *  - thread handles created by _beginthreadex (process.h), started by
 *    ResumeThread, identified by GetThreadId, joined by WaitForMultipleObjects
 *    (reference: pipeline.cpp PuresoftPipeline ctor/dtor, fragthrd.cpp
 *    fragmentThread thread-index lookup);
 *  - InterlockedIncrement/Decrement/Exchange on the ring-queue length
 *    (reference: rinque.h endPush/endPop);
 *  - the BMP header structs and _wfopen_s used by PuresoftFBO::saveAsBmpFile
 *    (reference: fbo.cpp), which the headless build never calls but must compile.
 * GetCurrentThread() returns a pseudo handle meaning "the calling thread", as
 * on Windows; GetThreadId() of it yields the caller's id.
 */
#pragma once
#include <stdint.h>
#include <stdio.h>
#include <wchar.h>
#include <stdlib.h>

typedef void* HANDLE;
typedef unsigned int DWORD;
typedef int BOOL;
typedef unsigned short WORD;
typedef int LONG;
#ifndef TRUE
#define TRUE 1
#endif
#ifndef FALSE
#define FALSE 0
#endif
#define INFINITE 0xFFFFFFFFu
#define CREATE_SUSPENDED 0x4u
#define BI_BITFIELDS 3

#ifdef __cplusplus
extern "C" {
#endif
HANDLE GetCurrentThread(void);
DWORD GetThreadId(HANDLE h);
DWORD ResumeThread(HANDLE h);
DWORD WaitForMultipleObjects(DWORD count, const HANDLE* handles, BOOL waitAll, DWORD ms);
BOOL CloseHandle(HANDLE h);
#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
template <class T> static inline T InterlockedIncrement(volatile T* p)
{
    return __atomic_add_fetch(p, (T)1, __ATOMIC_SEQ_CST);
}
template <class T> static inline T InterlockedDecrement(volatile T* p)
{
    return __atomic_sub_fetch(p, (T)1, __ATOMIC_SEQ_CST);
}
template <class T, class U> static inline T InterlockedExchange(volatile T* p, U v)
{
    return __atomic_exchange_n(p, (T)v, __ATOMIC_SEQ_CST);
}
#endif

#pragma pack(push, 2)
typedef struct {
    WORD bfType;
    DWORD bfSize;
    WORD bfReserved1;
    WORD bfReserved2;
    DWORD bfOffBits;
} BITMAPFILEHEADER;
#pragma pack(pop)

typedef struct {
    DWORD biSize;
    LONG biWidth;
    LONG biHeight;
    WORD biPlanes;
    WORD biBitCount;
    DWORD biCompression;
    DWORD biSizeImage;
    LONG biXPelsPerMeter;
    LONG biYPelsPerMeter;
    DWORD biClrUsed;
    DWORD biClrImportant;
} BITMAPINFOHEADER;

static inline int _wfopen_s(FILE** fp, const wchar_t* path, const wchar_t* mode)
{
    char p[4096], m[16];
    if (wcstombs(p, path, sizeof p) == (size_t)-1 || wcstombs(m, mode, sizeof m) == (size_t)-1) return 1;
    *fp = fopen(p, m);
    return *fp ? 0 : 1;
}
