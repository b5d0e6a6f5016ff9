// Host check of knnsj::exact_sqrt (csrc/exact_sqrt.cuh): every result must
// equal the C library's correctly rounded sqrt bit for bit.  Built and run by
// tests/test_exact_sqrt.py.
#include "exact_sqrt.cuh"
#include <cstdio>
#include <random>
int main() {
  std::mt19937_64 g(1);
  long bad = 0, n = 0;
  auto check = [&](double x) {
    double a = knnsj::exact_sqrt(x), b = std::sqrt(x);
    n++;
    if (std::memcmp(&a, &b, 8)) { if (bad < 5) printf("x=%a got %a want %a\n", x, a, b); bad++; }
  };
  for (int i = 0; i < 20000000; i++) {
    uint64_t bits = g() & 0x7fefffffffffffffull;  // positive finite
    double x; std::memcpy(&x, &bits, 8); check(x);
  }
  std::uniform_real_distribution<double> u(0, 1e4);
  for (int i = 0; i < 5000000; i++) check(u(g));
  for (int i = 0; i < 5000000; i++) { double s = (double)(g() >> 11); check(s * s); check(std::nextafter(s*s, 0)); check(std::nextafter(s*s, 1e300)); }
  for (int i = 0; i < 5000000; i++) { float a = (float)u(g), b = (float)u(g); check((double)(a*a) + (double)(b*b)); }
  // significands at both ends of [2^52, 2^53), both exponent parities: the
  // float seed's root reaches 2^27 at the top end
  for (int ex = 1; ex < 2047; ex += 7)
    for (uint64_t t = 0; t < 2000; t++) {
      for (uint64_t mant : {(uint64_t)((1ull << 52) - 1 - t), t}) {
        uint64_t bits = ((uint64_t)ex << 52) | mant;
        double x; std::memcpy(&x, &bits, 8); check(x);
      }
    }
  check(5e-324); check(1e-310); check(2.0); check(4.0); check(1.0); check(0x1.fffffffffffffp+1023);
  // the float-to-double conversion from bits, on every float bit pattern
  for (uint64_t fb = 0; fb < (1ull << 32); fb += 1 + (fb & 7)) {
    float f; uint32_t b32 = (uint32_t)fb; std::memcpy(&f, &b32, 4);
    double a = knnsj::es_f2d(f), c = (double)f;
    n++;
    if (std::memcmp(&a, &c, 8) && !(std::isnan(a) && std::isnan(c))) { if (bad < 5) printf("f=%a got %a\n", f, a); bad++; }
  }
  printf("n=%ld bad=%ld\n", n, bad);
  return bad != 0;
}
