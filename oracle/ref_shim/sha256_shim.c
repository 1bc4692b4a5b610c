/* Test infrastructure only: SHA256() for the reference binaries built by
 * oracle/ref.mk, implemented on top of bwo_sha256_hex (FIPS 180-4). */
#include <stddef.h>
#include "../bw_oracle.h"

unsigned char* SHA256(const unsigned char* d, size_t n, unsigned char* md) {
  char hex[65];
  bwo_sha256_hex(d, n, hex);
  for (int i = 0; i < 32; ++i) {
    int hi = hex[2 * i] <= '9' ? hex[2 * i] - '0' : hex[2 * i] - 'a' + 10;
    int lo = hex[2 * i + 1] <= '9' ? hex[2 * i + 1] - '0' : hex[2 * i + 1] - 'a' + 10;
    md[i] = (unsigned char)(hi * 16 + lo);
  }
  return md;
}
