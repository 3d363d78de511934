#include <cmath>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <random>
static inline double fixed_to_double(long long hi, long long lo, int e) {
  const __int128 v = ((__int128)hi << 28) + (__int128)lo;
  if (v == 0) return 0.0;
  const bool neg = v < 0;
  const unsigned __int128 m = neg ? (unsigned __int128)(-v) : (unsigned __int128)v;
  const unsigned long long mh = (unsigned long long)(m >> 64), ml = (unsigned long long)m;
  const int bl = mh ? 128 - __builtin_clzll(mh) : 64 - __builtin_clzll(ml);
  int sh = bl - 53;
  unsigned long long mant;
  if (sh <= 0) mant = (unsigned long long)(m << (-sh));
  else {
    unsigned __int128 q = m >> sh;
    const unsigned __int128 rem = m - (q << sh), half = (unsigned __int128)1 << (sh - 1);
    if (rem > half || (rem == half && (q & 1))) q += 1;
    if (q >> 53) { q >>= 1; sh += 1; }
    mant = (unsigned long long)q;
  }
  const int biased = sh + e - 63 + 52 + 1023;
  if (biased <= 0 || biased >= 2047) { const double d = ldexp((double)(long long)mant, sh + e - 63); return neg ? -d : d; }
  const unsigned long long bits = ((unsigned long long)neg << 63) | ((unsigned long long)biased << 52) | (mant & ((1ull << 52) - 1));
  double d; memcpy(&d, &bits, 8); return d;
}
// reference: exact via long double? use the ldexp sum (both exact inputs below 2^53 => one rounding)
int main() {
  std::mt19937_64 g(1);
  long bad = 0, n = 0;
  for (int it = 0; it < 2000000; ++it) {
    int hb = 1 + g() % 51, lb = 1 + g() % 51;
    long long hi = (long long)(g() >> (64 - hb)) * ((g() & 1) ? -1 : 1);
    long long lo = (long long)(g() >> (64 - lb)) * ((g() & 1) ? -1 : 1);
    if (it % 7 == 0) lo = (g() & 1) ? (1ll << 27) : -(1ll << 27);  // ties
    int e = (int)(g() % 200) - 100;
    double want = ldexp(ldexp((double)hi, -35) + ldexp((double)lo, -63), e);
    double got = fixed_to_double(hi, lo, e);
    ++n;
    if (memcmp(&want, &got, 8) != 0 && !(want == 0 && got == 0)) { if (bad < 5) printf("hi %lld lo %lld e %d want %.17g got %.17g\n", hi, lo, e, want, got); ++bad; }
  }
  // large-chunk sums: |hi| up to 2^51
  for (int it = 0; it < 200000; ++it) {
    long long hi = (long long)(g() >> 13) * ((g() & 1) ? -1 : 1), lo = (long long)(g() >> 13) * ((g() & 1) ? -1 : 1);
    double want = ldexp(ldexp((double)hi, -35) + ldexp((double)lo, -63), 3);
    double got = fixed_to_double(hi, lo, 3);
    ++n; if (memcmp(&want, &got, 8) != 0) { if (bad < 10) printf("B hi %lld lo %lld want %.17g got %.17g\n", hi, lo, want, got); ++bad; }
  }
  printf("%ld mismatches of %ld\n", bad, n);
}
