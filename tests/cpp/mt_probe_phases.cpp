// The device generator of Log_Det's probes (k_mt_probe in classicaldft_gb300/csrc/cdft_spectral.cu)
// restated on the host: std::mt19937's state twisted in three phases into a second copy
// (words i < 227 from old words; 227 <= i < 454 from the first phase's; the rest from the
// second phase's, word 623 also from the new word 0), each tempered word's top bit the
// draw, the state and the next unused word carried between calls. Compared draw for draw
// with std::mt19937(seed) and std::uniform_int_distribution<>(0, 1), over several calls of
// lengths that are not multiples of 624. Prints "ok" or the first mismatch.
#include <cstdio>
#include <random>
#include <vector>

static unsigned next_word(unsigned xi, unsigned xi1, unsigned xm) {
  const unsigned y = (xi & 0x80000000u) | (xi1 & 0x7fffffffu);
  return xm ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
}
static int draw_of(unsigned y) {
  y ^= y >> 11;
  y ^= (y << 7) & 0x9d2c5680u;
  y ^= (y << 15) & 0xefc60000u;
  y ^= y >> 18;
  return (int)(y >> 31);
}

struct PhaseGenerator {
  unsigned x[2][624];
  int cur = 0, pos = 624;
  explicit PhaseGenerator(unsigned long seed) {
    x[0][0] = (unsigned)seed;
    for (int i = 1; i < 624; ++i) x[0][i] = 1812433253u * (x[0][i - 1] ^ (x[0][i - 1] >> 30)) + (unsigned)i;
  }
  void draws(int* out, long n) {  // one k_mt_probe call
    long p = 0;
    for (; p < n && pos < 624; ++p) out[p] = draw_of(x[cur][pos++]);
    while (p < n) {
      const unsigned* o = x[cur];
      unsigned* nw = x[cur ^ 1];
      for (int t = 0; t < 227; ++t) nw[t] = next_word(o[t], o[t + 1], o[t + 397]);
      for (int t = 0; t < 227; ++t) nw[t + 227] = next_word(o[t + 227], o[t + 228], nw[t]);
      for (int t = 0; t < 169; ++t) nw[t + 454] = next_word(o[t + 454], o[t + 455], nw[t + 227]);
      nw[623] = next_word(o[623], nw[0], nw[396]);
      cur ^= 1;
      pos = 0;
      for (; p < n && pos < 624; ++p) out[p] = draw_of(x[cur][pos++]);
    }
  }
};

int main() {
  const long calls[] = {4096, 4096, 4096, 1000003, 624, 1, 623, 2097152};
  for (unsigned long seed : {1234ul, 77ul, 4321ul, 2024ul, 4294967295ul}) {
    std::mt19937 rng(seed);
    std::uniform_int_distribution<> d(0, 1);
    PhaseGenerator g(seed);
    long k = 0;
    for (long n : calls) {
      std::vector<int> a(n);
      g.draws(a.data(), n);
      for (long i = 0; i < n; ++i, ++k)
        if (a[i] != d(rng)) {
          std::printf("mismatch seed %lu draw %ld\n", seed, k);
          return 1;
        }
    }
  }
  std::printf("ok\n");
  return 0;
}
