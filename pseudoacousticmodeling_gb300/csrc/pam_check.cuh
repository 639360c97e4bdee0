// Bounds guard of the check build (compiled with -DPAM_BOUNDS_CHECK, see
// build.build_checked): an access of `bytes` bytes at p must lie inside
// [base, base + extent_bytes); otherwise the kernel prints the access site
// and offset and redirects the access to base, so that nothing outside the
// buffer is read or written.  In the normal build PAM_CHK(p, ...) is p.
#pragma once

#ifdef PAM_BOUNDS_CHECK
#include <cstdio>

namespace pam {
template <class T>
__device__ __forceinline__ T* pam_chk(T* p, const void* base, long long extent_bytes, int bytes, int site) {
    const char* c = reinterpret_cast<const char*>(p);
    const char* b = reinterpret_cast<const char*>(base);
    if (base == nullptr || c < b || c + bytes > b + extent_bytes) {
        printf("PAM_BOUNDS site %d offset %lld bytes %d extent %lld\n", site, (long long)(c - b), bytes,
               extent_bytes);
        return reinterpret_cast<T*>(const_cast<char*>(b));
    }
    return p;
}
}  // namespace pam
#define PAM_CHK(p, base, extent, bytes, site) pam::pam_chk((p), (base), (long long)(extent), (bytes), (site))
#else
#define PAM_CHK(p, base, extent, bytes, site) (p)
#endif
