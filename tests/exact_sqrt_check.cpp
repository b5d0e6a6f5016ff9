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
  check(5e-324); check(1e-310); check(2.0); check(4.0); check(1.0); check(0x1.fffffffffffffp+1023);
  printf("n=%ld bad=%ld\n", n, bad);
  return bad != 0;
}
