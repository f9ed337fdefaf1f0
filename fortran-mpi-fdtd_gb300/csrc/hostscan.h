// Host scans of a job's material-id grid (one byte per cell) at commit:
// the id histogram and the list of dispersive cells.  Both take eight cells
// per 64-bit word where the word allows it (a run of one id, or no
// dispersive id): a grid of millions of cells is mostly long runs of the
// background id.  Plain C++, no CUDA: the CPU tests compile it on its own.
#pragma once

#include <cstdint>
#include <cstring>

namespace fdtd {

// cnt[t] = number of cells with id t
inline void count_ids(const uint8_t *m, long long n, long long (&cnt)[256]) {
  // four interleaved sub-histograms for mixed words: runs of one id would
  // otherwise chain every increment on the same counter
  long long sub[4][256] = {};
  for (int t = 0; t < 256; ++t) cnt[t] = 0;
  const uint64_t ones = 0x0101010101010101ull;
  long long c = 0;
  for (; c + 8 <= n; c += 8) {
    uint64_t w;
    std::memcpy(&w, m + c, 8);
    const uint8_t b = m[c];
    if (w == ones * b) {  // eight cells of one id
      cnt[b] += 8;
      continue;
    }
    for (int u = 0; u < 8; ++u) sub[u & 3][m[c + u]]++;
  }
  for (; c < n; ++c) cnt[m[c]]++;
  for (int u = 0; u < 4; ++u)
    for (int t = 0; t < 256; ++t) cnt[t] += sub[u][t];
}

// f(c) for every cell c whose id has its high bit set (ids 128..255), in
// increasing order of c
template <typename F>
inline void for_high_ids(const uint8_t *m, long long n, F &&f) {
  long long c = 0;
  for (; c + 8 <= n; c += 8) {
    uint64_t w;
    std::memcpy(&w, m + c, 8);
    if (!(w & 0x8080808080808080ull)) continue;
    for (int u = 0; u < 8; ++u)
      if (m[c + u] & 0x80) f(c + u);
  }
  for (; c < n; ++c)
    if (m[c] & 0x80) f(c);
}

}  // namespace fdtd
