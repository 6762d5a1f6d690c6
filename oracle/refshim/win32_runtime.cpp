/*
 * win32_runtime.cpp -- runtime half of the Win32 stand-ins for the Linux build
 * of the reference pipeline core (oracle/_ref).  TEST INFRASTRUCTURE ONLY.
 *
 *  - _beginthreadex / ResumeThread / GetCurrentThread / GetThreadId /
 *    WaitForMultipleObjects / CloseHandle over pthreads (semantics as used by
 *    reference pipeline.cpp:55-61 and fragthrd.cpp:117-122);
 *  - logicCPUs(): the thread count the reference pipeline reads once into its
 *    static m_numberOfThreads (reference pipeline.cpp:17-22, cpu.cpp:23-72).
 *    Here it is PS3D_REF_THREADS if set, else std::thread::hardware_concurrency,
 *    never below 2 (with 1 thread the reference divides by zero in
 *    drawvao.cpp:83);
 *  - a headless PuresoftGdiRenderer: the class the reference declares in
 *    rndrgdi.h, implemented over two malloc'd BGRA buffers instead of GDI+, so
 *    that the reference's pipeline.cpp compiles and links unmodified;
 *  - mcemaths::align_base_16/64 operator new/delete (reference wraprs.cpp).
 */
#include <pthread.h>
#include <atomic>
#include <thread>
#include <new>
#include <string.h>
#include <stdlib.h>
#include "windows.h"
#include "process.h"
#include "mcemaths.hpp"
#include "rndrgdi.h"

namespace {

struct ThreadHandle {
    pthread_t th;
    unsigned (*fn)(void*);
    void* arg;
    DWORD id;
    bool started;
};

std::atomic<DWORD> g_nextId{1};
thread_local DWORD t_myId = 0;
HANDLE const kPseudoCurrent = (HANDLE)(intptr_t)-2;

DWORD currentId()
{
    if (!t_myId) t_myId = g_nextId.fetch_add(1);
    return t_myId;
}

void* trampoline(void* p)
{
    ThreadHandle* h = (ThreadHandle*)p;
    t_myId = h->id;
    h->fn(h->arg);
    return NULL;
}

} // namespace

extern "C" uintptr_t _beginthreadex(void*, unsigned, unsigned (*start)(void*), void* arg, unsigned flags, unsigned*)
{
    ThreadHandle* h = new ThreadHandle();
    h->fn = start;
    h->arg = arg;
    h->id = g_nextId.fetch_add(1);
    h->started = false;
    if (!(flags & CREATE_SUSPENDED)) ResumeThread((HANDLE)h);
    return (uintptr_t)h;
}

extern "C" DWORD ResumeThread(HANDLE hh)
{
    ThreadHandle* h = (ThreadHandle*)hh;
    if (h && !h->started) {
        h->started = true;
        if (pthread_create(&h->th, NULL, trampoline, h) != 0) abort();
    }
    return 0;
}

extern "C" HANDLE GetCurrentThread(void) { return kPseudoCurrent; }

extern "C" DWORD GetThreadId(HANDLE hh)
{
    if (hh == kPseudoCurrent) return currentId();
    return ((ThreadHandle*)hh)->id;
}

extern "C" DWORD WaitForMultipleObjects(DWORD count, const HANDLE* handles, BOOL, DWORD)
{
    for (DWORD i = 0; i < count; i++) {
        ThreadHandle* h = (ThreadHandle*)handles[i];
        if (h && h != kPseudoCurrent && h->started) {
            pthread_join(h->th, NULL);
            h->started = false;
        }
    }
    return 0;
}

extern "C" BOOL CloseHandle(HANDLE hh)
{
    if (hh && hh != kPseudoCurrent) delete (ThreadHandle*)hh;
    return TRUE;
}

int logicCPUs(void)
{
    const char* env = getenv("PS3D_REF_THREADS");
    int n = env ? atoi(env) : (int)std::thread::hardware_concurrency();
    return n < 2 ? 2 : n;
}

/* ---- headless renderer (stands in for GDI+ display) ---------------------- */

PuresoftGdiRenderer::PuresoftGdiRenderer(void)
    : m_width(0), m_height(0), m_canvasWindow(0), m_backBuffer(0), m_visibleBuffer(0),
      m_startRenderingEvent(0), m_renderingCompletionEvent(0), m_renderingThread(0)
{
    m_frameBuffers[0] = m_frameBuffers[1] = NULL;
}

PuresoftGdiRenderer::~PuresoftGdiRenderer(void) { destroyVisibleFBOs(); }

void PuresoftGdiRenderer::startup(uintptr_t canvasWindow, int width, int height)
{
    m_canvasWindow = canvasWindow;
    m_width = width;
    m_height = height;
    prepareVisibleFBOs();
}

void PuresoftGdiRenderer::shutdown(void) {}
void PuresoftGdiRenderer::setCanvas(uintptr_t canvasWindow) { m_canvasWindow = canvasWindow; }

void PuresoftGdiRenderer::getDesc(PURESOFTIMGBUFF32* desc)
{
    desc->width = m_width;
    desc->scanline = m_width * 4;
    desc->height = m_height;
    desc->elemLen = 4;
    desc->pixels = m_frameBuffers[m_backBuffer];
}

void* PuresoftGdiRenderer::swapBuffers(void)
{
    m_visibleBuffer = m_backBuffer;
    m_backBuffer = 1 - m_backBuffer;
    return m_frameBuffers[m_backBuffer];
}

void PuresoftGdiRenderer::release(void) { delete this; }

void PuresoftGdiRenderer::prepareVisibleFBOs(void)
{
    destroyVisibleFBOs();
    for (int i = 0; i < 2; i++) {
        m_frameBuffers[i] = _aligned_malloc((size_t)m_width * 4 * m_height, 64);
        memset(m_frameBuffers[i], 0, (size_t)m_width * 4 * m_height);
    }
}

void PuresoftGdiRenderer::destroyVisibleFBOs(void)
{
    for (int i = 0; i < 2; i++) {
        _aligned_free(m_frameBuffers[i]);
        m_frameBuffers[i] = NULL;
    }
}

unsigned PuresoftGdiRenderer::renderingThread(void*) { return 0; }

/* ---- mcemaths aligned allocation bases ----------------------------------- */

namespace mcemaths {
#define PS3D_ALIGNED_BASE(CLS, A)                                                        \
    void* CLS::operator new(size_t bytes)                                                \
    {                                                                                    \
        void* p = _aligned_malloc(bytes, A);                                             \
        if (!p) throw std::bad_alloc();                                                  \
        return p;                                                                        \
    }                                                                                    \
    void CLS::operator delete(void* mem) { _aligned_free(mem); }                         \
    void* CLS::operator new(size_t, void* place) { return place; }                       \
    void CLS::operator delete(void*, void*) {}                                           \
    void* CLS::operator new[](size_t bytes)                                              \
    {                                                                                    \
        void* p = _aligned_malloc(bytes, A);                                             \
        if (!p) throw std::bad_alloc();                                                  \
        return p;                                                                        \
    }                                                                                    \
    void CLS::operator delete[](void* mem) { _aligned_free(mem); }                       \
    void* CLS::operator new[](size_t, void* place) { return place; }                     \
    void CLS::operator delete[](void*, void*) {}
PS3D_ALIGNED_BASE(align_base_16, 16)
PS3D_ALIGNED_BASE(align_base_64, 64)
} // namespace mcemaths
