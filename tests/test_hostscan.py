"""The commit's word-level scans of the material-id grid (csrc/hostscan.h)
against byte-by-byte scans, on CPU: grids of runs, random ids, dispersive ids
at word edges, and lengths that are not a multiple of eight."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "fortran-mpi-fdtd_gb300", "csrc")

DRIVER = r"""
#include <cstdio>
#include <vector>
#include "hostscan.h"
using namespace fdtd;
static unsigned long long s = 12345;
static unsigned rnd() { s = s * 6364136223846793005ull + 1442695040888963407ull; return (unsigned)(s >> 33); }
int check(const std::vector<uint8_t> &m) {
  const long long n = (long long)m.size();
  long long ref[256] = {}, got[256];
  std::vector<long long> hr, hg;
  for (long long c = 0; c < n; ++c) {
    ref[m[c]]++;
    if (m[c] >= 128) hr.push_back(c);
  }
  count_ids(m.data(), n, got);
  for_high_ids(m.data(), n, [&](long long c) { hg.push_back(c); });
  for (int t = 0; t < 256; ++t)
    if (ref[t] != got[t]) { printf("count mismatch n=%lld id=%d %lld %lld\n", n, t, ref[t], got[t]); return 1; }
  if (hr != hg) { printf("dispersive list mismatch n=%lld %zu %zu\n", n, hr.size(), hg.size()); return 1; }
  return 0;
}
int main() {
  int bad = 0;
  for (long long n : {0LL, 1LL, 7LL, 8LL, 9LL, 63LL, 64LL, 1000LL, 4099LL, 100003LL}) {
    std::vector<uint8_t> m(n);
    for (auto &x : m) x = (uint8_t)rnd();                      // random ids
    bad |= check(m);
    for (long long c = 0; c < n; ++c) m[c] = (uint8_t)((c / 37) % 3);  // runs of a few ids
    bad |= check(m);
    for (auto &x : m) x = 5;                                   // one id
    for (long long c = 7; c < n; c += 61) m[c] = 130;          // dispersive ids at scattered places
    for (long long c = 8; c < n; c += 64) m[c] = 255;          // ... and at word starts
    bad |= check(m);
    for (long long c = 0; c < n; ++c) m[c] = (uint8_t)(rnd() % 1000 < 3 ? 128 + rnd() % 128 : 1);
    bad |= check(m);
  }
  printf(bad ? "FAIL\n" : "ok\n");
  return bad;
}
"""


def test_word_scans_match_byte_scans(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if not cxx:
        pytest.skip("no C++ compiler")
    src = tmp_path / "scan.cpp"
    exe = tmp_path / "scan"
    src.write_text(DRIVER)
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", CSRC, str(src), "-o", str(exe)], check=True, timeout=120)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
