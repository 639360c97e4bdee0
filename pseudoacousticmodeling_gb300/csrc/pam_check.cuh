// Bounds guard of the check build (compiled with -DPAM_BOUNDS_CHECK, see
// build.build_checked): an access of `bytes` bytes at p must lie inside
// [base, base + extent_bytes) of a non-null base; otherwise the kernel prints
// the access site and offset and redirects the access to a small scratch
// array of the check build, so that nothing outside the buffer is read or
// written, whether or not the buffer exists.  In the normal build
// PAM_CHK(p, ...) is p.
#pragma once

#ifdef PAM_BOUNDS_CHECK
#include <cstdio>

namespace pam {
// target of every redirected access (the widest guarded access is 36 bytes);
// one copy per translation unit
static __device__ __align__(16) unsigned char g_chk_scratch[256];

template <class T>
__device__ __forceinline__ T* pam_chk(T* p, const void* base, long long extent_bytes, int bytes, int site) {
    const char* c = reinterpret_cast<const char*>(p);
    const char* b = reinterpret_cast<const char*>(base);
    if (base == nullptr || c < b || c + bytes > b + extent_bytes) {
        printf("PAM_BOUNDS site %d offset %lld bytes %d extent %lld\n", site, (long long)(c - b), bytes,
               extent_bytes);
        return reinterpret_cast<T*>(g_chk_scratch);
    }
    return p;
}
}  // namespace pam
#define PAM_CHK(p, base, extent, bytes, site) pam::pam_chk((p), (base), (long long)(extent), (bytes), (site))
#else
#define PAM_CHK(p, base, extent, bytes, site) (p)
#endif
