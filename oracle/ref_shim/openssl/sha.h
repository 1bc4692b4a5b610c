/* Minimal stand-in for the one OpenSSL entry point the reference's timed workers
 * call (sha_fast.hpp:30).  The OpenSSL headers are absent from this image; the
 * definition lives in oracle/ref_shim/sha256_shim.c and forwards to the oracle's
 * own FIPS 180-4 implementation.  Test infrastructure only. */
#pragma once
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
unsigned char* SHA256(const unsigned char* d, size_t n, unsigned char* md);
#ifdef __cplusplus
}
#endif
