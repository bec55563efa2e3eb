/* Which C-library pow a host has: pow over a deterministic sample of exactly
   constructed inputs (splitmix64 bits for the mantissa and the binade; no
   libm call makes them) for the exponents of the reference's DOP853 step
   controller (-1/9, 0.4/9, -1/8) and variational Jacobian (1.5, 2.5); prints
   "exponent chunk hash", one FNV-1a hash of the result bits per chunk of 10^6
   calls.  Two hosts whose outputs match return the same bits on every sample.
   Build: gcc -O2 -fno-builtin -o libm_pow_hash libm_pow_hash.c -lm
   Run:   ./libm_pow_hash 100 > hashes.txt */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

static uint64_t s;
static uint64_t next_bits(void) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

int main(int argc, char** argv) {
  const long chunks = argc > 1 ? atol(argv[1]) : 100;
  const double ys[5] = {-1.0 / 9.0, 0.4 / 9.0, -1.0 / 8.0, 1.5, 2.5};
  for (int k = 0; k < 5; k++) {
    s = 0x9E3779B97F4A7C15ull + k;
    for (long c = 0; c < chunks; c++) {
      uint64_t h = 1469598103934665603ull;
      for (long i = 0; i < 1000000; i++) {
        const uint64_t b = next_bits();
        const int e = k < 3 ? -40 + (int)(b % 45) : -6 + (int)(b % 12);
        const double x = ldexp(1.0 + (double)(b >> 12) * 0x1p-52, e);
        const double r = pow(x, ys[k]);
        uint64_t rb;
        memcpy(&rb, &r, 8);
        h = (h ^ rb) * 1099511628211ull;
      }
      printf("%d %ld %016llx\n", k, c, (unsigned long long)h);
    }
  }
  return 0;
}
