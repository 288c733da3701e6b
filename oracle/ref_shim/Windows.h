/* POSIX stand-ins for the Win32 calls the Origami reference headers use, so the
 * reference can be compiled unmodified with g++ on Linux (test infrastructure:
 * only the oracle recipe in oracle/Makefile puts this directory on the include
 * path). Each definition maps one Win32 name onto pthreads / libc. */
#pragma once
#include <pthread.h>
#include <sched.h>
#include <stdlib.h>
#include <string.h>
#include <stdint.h>
#include <type_traits>

#define FORCEINLINE inline
#define __declspec(x) __attribute__((x))
typedef long long __int64;
typedef unsigned long DWORD;
typedef int BOOL;
#define TRUE 1
#define FALSE 0
#define INFINITE 0xFFFFFFFFu

/* two-argument min/max as provided by <windows.h> (the reference mixes types) */
template <class A, class B>
inline typename std::common_type<A, B>::type min(A a, B b) { return b < a ? b : a; }
template <class A, class B>
inline typename std::common_type<A, B>::type max(A a, B b) { return a < b ? b : a; }

/* VirtualAlloc/VirtualFree: page-aligned, zero-initialised like the Win32 call */
#define MEM_COMMIT 0x1000
#define MEM_RESERVE 0x2000
#define MEM_RELEASE 0x8000
#define PAGE_READWRITE 0x04
inline void* VirtualAlloc(void*, size_t sz, int, int) {
    void* p = nullptr;
    if (posix_memalign(&p, 4096, sz ? sz : 4096) != 0) return nullptr;
    memset(p, 0, sz);
    return p;
}
inline BOOL VirtualFree(void* p, size_t, int) { free(p); return TRUE; }

/* critical sections -> mutexes */
typedef pthread_mutex_t CRITICAL_SECTION;
inline void InitializeCriticalSection(CRITICAL_SECTION* c) { pthread_mutex_init(c, nullptr); }
inline void EnterCriticalSection(CRITICAL_SECTION* c) { pthread_mutex_lock(c); }
inline void LeaveCriticalSection(CRITICAL_SECTION* c) { pthread_mutex_unlock(c); }
inline void DeleteCriticalSection(CRITICAL_SECTION* c) { pthread_mutex_destroy(c); }

/* synchronization barrier -> pthread barrier */
typedef pthread_barrier_t SYNCHRONIZATION_BARRIER;
#define SYNCHRONIZATION_BARRIER_FLAGS_BLOCK_ONLY 1
inline BOOL InitializeSynchronizationBarrier(SYNCHRONIZATION_BARRIER* b, long n, long) {
    return pthread_barrier_init(b, nullptr, (unsigned)n) == 0;
}
inline BOOL EnterSynchronizationBarrier(SYNCHRONIZATION_BARRIER* b, DWORD) {
    pthread_barrier_wait(b);
    return FALSE;
}
inline BOOL DeleteSynchronizationBarrier(SYNCHRONIZATION_BARRIER* b) {
    pthread_barrier_destroy(b);
    return TRUE;
}

/* manual-reset / auto-reset events -> mutex + condition variable */
struct OrigamiShimEvent {
    pthread_mutex_t m;
    pthread_cond_t c;
    int signaled;
    int manual;
};
typedef OrigamiShimEvent* HANDLE;
inline HANDLE CreateEvent(void*, BOOL manual, BOOL initial, const char*) {
    HANDLE h = new OrigamiShimEvent;
    pthread_mutex_init(&h->m, nullptr);
    pthread_cond_init(&h->c, nullptr);
    h->signaled = initial ? 1 : 0;
    h->manual = manual ? 1 : 0;
    return h;
}
inline BOOL SetEvent(HANDLE h) {
    pthread_mutex_lock(&h->m);
    h->signaled = 1;
    pthread_cond_broadcast(&h->c);
    pthread_mutex_unlock(&h->m);
    return TRUE;
}
inline DWORD WaitForSingleObject(HANDLE h, DWORD) {
    pthread_mutex_lock(&h->m);
    while (!h->signaled) pthread_cond_wait(&h->c, &h->m);
    if (!h->manual) h->signaled = 0;
    pthread_mutex_unlock(&h->m);
    return 0;
}

inline BOOL CloseHandle(HANDLE h) {
    pthread_cond_destroy(&h->c);
    pthread_mutex_destroy(&h->m);
    delete h;
    return TRUE;
}

inline long long InterlockedIncrement64(volatile long long* p) {
    return __atomic_add_fetch(p, 1, __ATOMIC_SEQ_CST);
}
inline BOOL SwitchToThread() { return sched_yield() == 0; }
inline void* GetCurrentThread() { return nullptr; }
template <class H, class M>
inline uintptr_t SetThreadAffinityMask(H, M) { return 1; }

inline int strcat_s(char* dst, size_t n, const char* src) {
    strncat(dst, src, n - strlen(dst) - 1);
    return 0;
}
