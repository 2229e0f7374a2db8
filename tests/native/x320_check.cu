// Host-side check of the exact-sum helpers in amcl3d_gb300/csrc/exact.cuh: reads
// 320-bit two's-complement values (5 hex words, least significant first) and prints
// the double each converts to, plus any digit-split round-trip failure.
#include <cstdio>
#include <cinttypes>
#include "../../amcl3d_gb300/csrc/exact.cuh"
using namespace amcl;
int main(){
  unsigned long long w[5];
  while (scanf("%llx %llx %llx %llx %llx", &w[0],&w[1],&w[2],&w[3],&w[4]) == 5) {
    X320 a; for (int i=0;i<5;++i) a.w[i]=w[i];
    printf("%a\n", x320_to_double(a));
    // digits roundtrip
    unsigned long long d[10];
    for (int j=0;j<10;++j){ uint64_t word=a.w[j>>1]; uint64_t dig=(j&1)?(word>>32):(word&0xFFFFFFFFull); if(j==9) dig=(uint64_t)(int64_t)(int32_t)(uint32_t)dig; d[j]=dig; }
    X320 b = x320_from_digits(d);
    for (int i=0;i<5;++i) if (b.w[i]!=a.w[i]) { printf("DIGITS MISMATCH\n"); break; }
  }
}
