// Host check of arcanefem_gb300/csrc/afem_fp64_int.cuh against the host's
// IEEE binary64 add, subtract and multiply (test infrastructure).
//   fp64_int_check <pairs> <seed>  ->  prints "mismatches mul add sub fallbacks"
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "afem_fp64_int.cuh"

static uint64_t st;
static uint64_t next() {
  st ^= st << 13;
  st ^= st >> 7;
  st ^= st << 17;
  return st;
}

int main(int argc, char** argv) {
  const long n = argc > 1 ? atol(argv[1]) : 1000000;
  st = argc > 2 ? strtoull(argv[2], nullptr, 10) : 88172645463325252ull;
  long bad_mul = 0, bad_add = 0, bad_sub = 0, fallbacks = 0;
  for (long i = 0; i < n; ++i) {
    uint64_t a = next(), b = next();
    const int mode = (int)(i % 6);
    const int ea = 1023 + (int)(next() % 80) - 40;
    int eb = mode == 0 ? 1023 + (int)(next() % 160) - 80 : ea + (int)(next() % (mode == 1 ? 3 : 70)) - (mode == 1 ? 1 : 35);
    if (eb < 1) eb = 1;
    a = (a & ~(0x7ffull << 52)) | ((uint64_t)ea << 52);
    b = (b & ~(0x7ffull << 52)) | ((uint64_t)eb << 52);
    if (mode == 3) b = ((a & ~(1ull << 63)) ^ (next() & 0xff)) | (b & (1ull << 63));   // near-equal magnitudes
    if (mode == 4) b |= 0xFFFFFFFFFFFF0ull;                                            // significand near 2
    if (mode == 5 && (i & 16)) b = a ^ (1ull << 63);                                   // exact cancellation
    double da, db;
    std::memcpy(&da, &a, 8);
    std::memcpy(&db, &b, 8);
    const double hm = da * db, ha = da + db, hs = da - db;
    uint64_t um, ua_, us, r;
    std::memcpy(&um, &hm, 8);
    std::memcpy(&ua_, &ha, 8);
    std::memcpy(&us, &hs, 8);
    if (afem::i64fp::mul(a, b, &r)) bad_mul += r != um; else ++fallbacks;
    if (afem::i64fp::add(a, b, &r)) bad_add += r != ua_; else ++fallbacks;
    if (afem::i64fp::add(a, b ^ (1ull << 63), &r)) bad_sub += r != us; else ++fallbacks;
  }
  std::printf("%ld %ld %ld %ld\n", bad_mul, bad_add, bad_sub, fallbacks);
  return 0;
}
