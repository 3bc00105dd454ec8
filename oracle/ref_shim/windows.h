/*
 * ORACLE — test infrastructure only.  The subset of <windows.h> that the
 * reference's src/dsp_plugin.c, src/engine.c and src/fir.c name, stated on
 * POSIX so those files compile where they lie (oracle/Makefile, target ref).
 * Threads, events and CPU sets are not needed: the harness runs the plugin's
 * thread-pool blocks inline (oracle/ref_plugin.c).  Timers read
 * CLOCK_MONOTONIC; atomics are the GCC builtins.
 */
#ifndef ORACLE_REF_WINDOWS_H
#define ORACLE_REF_WINDOWS_H

#include <stdint.h>
#include <stddef.h>
#include <time.h>
#include <unistd.h>
#include <wchar.h>

typedef int BOOL;
typedef int32_t LONG;
typedef uint32_t ULONG;
typedef unsigned long DWORD;
typedef uintptr_t DWORD_PTR;
typedef uint64_t ULONGLONG;
typedef int64_t LONGLONG;
typedef void *HANDLE;
typedef void *HMODULE;
typedef void *LPVOID;
typedef void *PVOID;
typedef unsigned short WORD;
typedef unsigned char BYTE;
typedef struct { void *p; } SRWLOCK;
typedef struct { void *p; } CRITICAL_SECTION;
typedef union {
    struct { DWORD LowPart; LONG HighPart; } u;
    LONGLONG QuadPart;
} LARGE_INTEGER;

#define TRUE 1
#define FALSE 0
#define WINAPI
#define MAX_PATH 260
#define INFINITE 0xFFFFFFFFu
#define ES_CONTINUOUS 0x80000000u
#define ES_SYSTEM_REQUIRED 0x00000001u
#define SRWLOCK_INIT {0}

/* __declspec(thread) -> __thread; __declspec(align(n)) -> aligned(n) */
#define __declspec(x) __declspec_##x
#define __declspec_thread __thread
#define __declspec_dllexport
#define __declspec_noinline __attribute__((noinline))
#define __declspec_align(n) __attribute__((aligned(n)))

static inline BOOL QueryPerformanceCounter(LARGE_INTEGER *t)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    t->QuadPart = (LONGLONG)ts.tv_sec * 1000000000LL + ts.tv_nsec;
    return TRUE;
}
static inline BOOL QueryPerformanceFrequency(LARGE_INTEGER *f)
{
    f->QuadPart = 1000000000LL;
    return TRUE;
}
static inline void Sleep(DWORD ms) { usleep((useconds_t)ms * 1000u); }
static inline DWORD GetTickCount(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (DWORD)(ts.tv_sec * 1000 + ts.tv_nsec / 1000000);
}
static inline ULONGLONG GetTickCount64(void) { return GetTickCount(); }
static inline HMODULE GetModuleHandleA(const char *n) { (void)n; return NULL; }
static inline HMODULE GetModuleHandleW(const wchar_t *n) { (void)n; return NULL; }
static inline void *GetProcAddress(HMODULE m, const char *n) { (void)m; (void)n; return NULL; }
static inline DWORD GetModuleFileNameW(HMODULE m, wchar_t *b, DWORD n)
{
    (void)m;
    if (n) b[0] = 0;
    return 0;
}
static inline DWORD SetThreadExecutionState(DWORD f) { (void)f; return 0; }
static inline void InitializeSRWLock(SRWLOCK *l) { l->p = NULL; }
static inline void AcquireSRWLockExclusive(SRWLOCK *l) { (void)l; }
static inline void ReleaseSRWLockExclusive(SRWLOCK *l) { (void)l; }
static inline void AcquireSRWLockShared(SRWLOCK *l) { (void)l; }
static inline void ReleaseSRWLockShared(SRWLOCK *l) { (void)l; }
static inline void InitializeCriticalSection(CRITICAL_SECTION *c) { c->p = NULL; }
static inline void DeleteCriticalSection(CRITICAL_SECTION *c) { (void)c; }
static inline void EnterCriticalSection(CRITICAL_SECTION *c) { (void)c; }
static inline void LeaveCriticalSection(CRITICAL_SECTION *c) { (void)c; }
static inline LONG InterlockedCompareExchange(volatile LONG *d, LONG x, LONG c)
{
    return __sync_val_compare_and_swap(d, c, x);
}
static inline LONG InterlockedExchange(volatile LONG *d, LONG x) { return __sync_lock_test_and_set(d, x); }
static inline LONG InterlockedIncrement(volatile LONG *d) { return __sync_add_and_fetch(d, 1); }
static inline LONG InterlockedDecrement(volatile LONG *d) { return __sync_sub_and_fetch(d, 1); }
static inline void OutputDebugStringA(const char *s) { (void)s; }
static inline DWORD GetLastError(void) { return 0; }
static inline BOOL CloseHandle(HANDLE h) { (void)h; return TRUE; }
static inline DWORD GetCurrentProcessorNumber(void) { return 0; }

#define INVALID_FILE_ATTRIBUTES 0xFFFFFFFFu
static inline DWORD GetFileAttributesW(const wchar_t *p) { (void)p; return INVALID_FILE_ATTRIBUTES; }
static inline DWORD GetFileAttributesA(const char *p) { (void)p; return INVALID_FILE_ATTRIBUTES; }

/* the plugin's log sink (defined by the harness) */
void trellis_log_c(const char *msg);

#define sprintf_s snprintf
#define _snprintf snprintf

#endif
