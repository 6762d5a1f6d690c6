/*
 * process.h stand-in (oracle/_ref, TEST INFRASTRUCTURE ONLY): _beginthreadex.
 * The thread is created suspended in the Windows sense: it starts running only
 * when ResumeThread is called on the returned handle, which is what the
 * reference's PuresoftPipeline constructor relies on (it stores the handle in
 * m_threads[] before resuming, and fragmentThread looks its own index up
 * there).
 */
#pragma once
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif
uintptr_t _beginthreadex(void* security, unsigned stackSize, unsigned (*start)(void*), void* arg,
                         unsigned initFlags, unsigned* threadAddr);
#ifdef __cplusplus
}
#endif
