// Host harness for lightgraphs.jl_gb300/csrc/xf64.cuh (compiled by
// tests/test_xf64_host.py with g++).  Reads commands from stdin, one per line:
//   R s            -> reciprocal of the integer s
//   M a_bits s     -> (double a) * s
//   A a_bits b_bits -> double a + double b
//   X a_bits b_bits -> double a * double b
//   S n b1 .. bn   -> sum of n doubles, accumulated term by term
//   G n b1 .. bn   -> the same with the gather accumulator (xg64)
// and prints, per line, the result as "m e bits" (xf64 and its binary64 rounding).
#include <cstdio>
#include <cstring>
#include "xf64.cuh"

using namespace lgbc;

int main() {
  char op[4];
  while (std::scanf("%3s", op) == 1) {
    xf64 r{};
    if (op[0] == 'R') {
      unsigned long long s;
      std::scanf("%llu", &s);
      r = xf_recip_u64(s);
    } else if (op[0] == 'M') {
      unsigned long long a, s;
      std::scanf("%llu %llu", &a, &s);
      r = xf_mul_u64(xf_from_bits(a), s);
    } else if (op[0] == 'A') {
      unsigned long long a, b;
      std::scanf("%llu %llu", &a, &b);
      r = xf_add(xf_from_bits(a), xf_from_bits(b));
    } else if (op[0] == 'X') {
      unsigned long long a, b;
      std::scanf("%llu %llu", &a, &b);
      r = xf_mul(xf_from_bits(a), xf_from_bits(b));
    } else if (op[0] == 'G') {
      // G n b1 .. bn: the gather accumulator, renormalised every 32 terms
      int n;
      std::scanf("%d", &n);
      xg64 g = xg_zero();
      for (int i = 0; i < n; ++i) {
        unsigned long long b;
        std::scanf("%llu", &b);
        xg_add_bits(g, b);
        if (i % 32 == 31) xg_norm(g);
      }
      xg_norm(g);
      r = xg_to_xf(g);
    } else if (op[0] == 'S') {
      int n;
      std::scanf("%d", &n);
      r = xf_zero();
      for (int i = 0; i < n; ++i) {
        unsigned long long b;
        std::scanf("%llu", &b);
        r = xf_add_bits(r, b);
      }
    }
    std::printf("%llu %d %llu\n", static_cast<unsigned long long>(r.m), r.e,
                static_cast<unsigned long long>(xf_to_bits(r)));
  }
  return 0;
}
