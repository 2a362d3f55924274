// Host check of exact_to_double (slakonet_gb300/csrc/exact_round.cuh): against the FP64 expression it
// replaces in the tensor-core update's epilogue, bit for bit, on random level sums in the ranges the update
// produces, near-ties and exponent edges.  Prints the mismatch count.  (Where 2^(e + 56) itself overflows,
// the expression gives inf and exact_to_double the finite value; the update's exponents never get there.)
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>

#include "exact_round.cuh"

int main(int argc, char** argv) {
  const long long cases = argc > 1 ? atoll(argv[1]) : 2000000;
  std::mt19937_64 g(20261204);
  long long bad = 0;
  for (long long it = 0; it < cases; ++it) {
    long long hi = (long long)(g() >> 14) - (1ll << 49);      // |hi| < 2^50
    long long lo = (long long)(g() >> 20) - (1ll << 43);      // |lo| < 2^44
    switch (it % 5) {
      case 1: hi >>= (g() % 50); break;                        // all magnitudes
      case 2: hi = 0; lo >>= (g() % 44); break;                // low half alone
      case 3: lo = (long long)((int)(g() % 3) - 1) << (g() % 21); break;   // halfway and near-halfway sums
      case 4: hi = -hi; lo = -lo; break;
      default: break;
    }
    // exponents that keep the reference's scale factor 2^(e + 56) a normal double (the kernel's are near
    // 0), with results reaching into the subnormal and overflow ranges
    const int e = (int)(g() % 2030) - 1070;
    const double ref = std::fma((double)hi, 0x1p-35, (double)lo * 0x1p-56) * std::ldexp(1.0, e + 56);
    const double got = exact_to_double(hi, lo, e);
    if (std::memcmp(&ref, &got, sizeof ref) != 0) {
      if (bad < 5) std::printf("hi=%lld lo=%lld e=%d: expected %.17g, got %.17g\n", hi, lo, e, ref, got);
      ++bad;
    }
  }
  std::printf("%lld mismatches in %lld cases\n", bad, cases);
  return bad != 0;
}
