// Reads lines "op a b q" from stdin and prints the result of heal_arith.h's
// routine for them, so tests/test_arith.py can compare with Python integers.
#include <cstdio>
#include <cstring>
#include "../../heal_gb300/csrc/heal_arith.h"
using namespace heal;
int main() {
  char op[16];
  unsigned long long a, b, q;
  while (scanf("%15s %llu %llu %llu", op, &a, &b, &q) == 4) {
    unsigned long long r = 0;
    if (!strcmp(op, "mul64")) r = mg64_mulmod(a, b, mg64_make((int64_t)q));
    else if (!strcmp(op, "mod128")) r = mg64_mod(a, b, mg64_make((int64_t)q));
    else if (!strcmp(op, "mod32")) r = mg32_mod(((uint64_t)a << 32) | b, mg32_make((int64_t)q));
    else if (!strcmp(op, "shoup64")) r = shoup64(a, b, shoup64_companion(b, q), q);
    else if (!strcmp(op, "shoup32")) r = shoup32((uint32_t)a, (uint32_t)b, shoup32_companion((uint32_t)b, (uint32_t)q), (uint32_t)q);
    else if (!strcmp(op, "fastdiv")) r = fastdiv((uint32_t)a, fastdiv_make((uint32_t)q));
    printf("%llu\n", r);
  }
  return 0;
}
