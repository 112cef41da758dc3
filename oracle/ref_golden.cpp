/*
 * ref_golden.cpp -- golden vectors from the reference's own random.hpp.
 *
 * TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile (target `ref`) against
 * the reference source tree, which must be on the include path; the binary
 * lands in oracle/_ref/.  random.hpp needs nothing but the
 * KOKKOS_INLINE_FUNCTION macro, which the recipe defines as `inline`.
 *
 * Output (stdout, JSON):
 *  - "lcg": dRandom sequences (random.hpp:87) for a few seeds: 64-bit rand()
 *    values and the bit patterns of drand() values;
 *  - "fill": for (elem, ipart, type, n_global_elem) tuples, the seed of
 *    particle_fill.hpp:147, the 10 burned draws, and the accepted x_ref of the
 *    rejection loop of particle_fill.hpp:152-156 (bit patterns).
 * The seed expression is restated here with the reference's operand types
 * (LO elem, size_t ipart, GO n_global_elem, int type).
 */
#include <cstdio>
#include <cstdint>
#include <cstring>
#include "random.hpp"

static unsigned long long bits(double d) {
  unsigned long long u;
  memcpy(&u, &d, 8);
  return u;
}

int main() {
  printf("{\n  \"lcg\": [\n");
  const unsigned long seeds[] = {0UL, 1UL, 12345UL, 34030UL * 6000UL, 18446744073709551615UL};
  const int ns = sizeof(seeds) / sizeof(seeds[0]);
  for (int s = 0; s < ns; ++s) {
    dRandom r;
    r.srand(seeds[s]);
    printf("    {\"seed\": %lu, \"rand\": [", seeds[s]);
    for (int i = 0; i < 8; ++i) printf("%s%lu", i ? ", " : "", r.rand());
    dRandom r2;
    r2.srand(seeds[s]);
    printf("], \"drand_bits\": [");
    for (int i = 0; i < 8; ++i) printf("%s%llu", i ? ", " : "", bits(r2.drand()));
    printf("]}%s\n", s + 1 < ns ? "," : "");
  }
  printf("  ],\n  \"fill\": [\n");
  struct Case { int elem; size_t ipart; long ng; int type; };
  const Case cases[] = {{0, 0, 6000, 0}, {17, 3, 6000, 0}, {5999, 9, 6000, 1}, {123, 1, 5000, 2},
                        {4999, 0, 5000, 0}, {0, 99, 40, 1}, {39, 7, 40, 0}};
  const int nc = sizeof(cases) / sizeof(cases[0]);
  for (int c = 0; c < nc; ++c) {
    const int elem = cases[c].elem;
    const size_t ipart = cases[c].ipart;
    const long n_global_elem = cases[c].ng;
    const int type_ = cases[c].type;
    dRandom rnd;
    unsigned long seed = elem + (34030 + ipart) * n_global_elem + n_global_elem * 12345 * type_;
    rnd.srand(seed);
    for (int i = 0; i < 10; ++i) rnd.rand();
    double x0, x1, x2;
    int tries = 0;
    do {
      x0 = rnd.drand();
      x1 = rnd.drand();
      x2 = rnd.drand();
      ++tries;
    } while (x0 + x1 + x2 > 1.0);
    printf("    {\"elem\": %d, \"ipart\": %zu, \"n_global_elem\": %ld, \"type\": %d, \"seed\": %lu, "
           "\"tries\": %d, \"xref_bits\": [%llu, %llu, %llu]}%s\n",
           elem, ipart, n_global_elem, type_, seed, tries, bits(x0), bits(x1), bits(x2), c + 1 < nc ? "," : "");
  }
  printf("  ]\n}\n");
  return 0;
}
