/* Minimal stand-in for the few Win32 thread calls the reference renderer
 * makes (thread priority and thread id).  Test infrastructure only: it lets
 * the reference sources compile with g++ so they can serve as the oracle. */
#ifndef SKW_REF_SHIM_WINDOWS_H
#define SKW_REF_SHIM_WINDOWS_H

#include <unistd.h>
#include <sys/syscall.h>

typedef void *HANDLE;
#define THREAD_PRIORITY_LOWEST (-2)
#define THREAD_PRIORITY_NORMAL 0

inline HANDLE GetCurrentThread() { return (HANDLE)0; }
inline int GetThreadPriority(HANDLE) { return THREAD_PRIORITY_NORMAL; }
inline int SetThreadPriority(HANDLE, int) { return 1; }
inline unsigned long GetCurrentThreadId() { return (unsigned long)syscall(SYS_gettid); }

#endif
