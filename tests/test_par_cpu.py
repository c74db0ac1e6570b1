"""The build's parallel host passes (hodlrnd_gb300/csrc/par.h): the prefix sums
and the per-operator running offsets that place every far block's descriptor
and factor bytes, checked against their sequential definitions on the host
for sizes below and above the one-thread cut-off, with several thread counts.
"""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "hodlrnd_gb300", "csrc")

PROGRAM = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "par.h"

using namespace hodlr;

static uint64_t mix(uint64_t v) {  // a fixed pseudo-random sequence
  v += 0x9E3779B97F4A7C15ull;
  v = (v ^ (v >> 30)) * 0xBF58476D1CE4E5B9ull;
  v = (v ^ (v >> 27)) * 0x94D049BB133111EBull;
  return v ^ (v >> 31);
}

int main() {
  const int64_t sizes[] = {0, 1, 7, 65535, 65536, 65537, 1000003};
  int bad = 0;
  for (int64_t n : sizes) {
    std::vector<uint64_t> val(static_cast<size_t>(n)), scan(static_cast<size_t>(n) + 1);
    for (int64_t i = 0; i < n; i++) val[size_t(i)] = mix(uint64_t(i)) % 1000;
    par_exclusive_scan(n, scan.data(), [&](int64_t i) { return val[size_t(i)]; });
    uint64_t s = 0;
    for (int64_t i = 0; i < n; i++) {
      if (scan[size_t(i)] != s) bad++;
      s += val[size_t(i)];
    }
    if (scan[size_t(n)] != s) bad++;
    for (int groups : {1, 3, 256}) {
      std::vector<int> grp(static_cast<size_t>(n));
      for (int64_t i = 0; i < n; i++) grp[size_t(i)] = int(mix(uint64_t(i) + 7) % uint64_t(groups));
      std::vector<uint64_t> off(static_cast<size_t>(n)), total;
      par_group_offsets(
          n, groups, off.data(), total, [&](int64_t i) { return grp[size_t(i)]; },
          [&](int64_t i) { return val[size_t(i)]; });
      std::vector<uint64_t> run(static_cast<size_t>(groups), 0);
      for (int64_t i = 0; i < n; i++) {
        const int g = grp[size_t(i)];
        if (off[size_t(i)] != run[size_t(g)]) bad++;
        run[size_t(g)] += val[size_t(i)];
      }
      if (total.size() != size_t(groups)) {
        bad++;
      } else {
        for (int g = 0; g < groups; g++)
          if (total[size_t(g)] != run[size_t(g)]) bad++;
      }
    }
  }
  std::printf("%d\n", bad);
  return bad == 0 ? 0 : 1;
}
"""


@pytest.mark.parametrize("threads", [1, 3, 8])
def test_parallel_scans_match_sequential(tmp_path, threads):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    src = tmp_path / "par_check.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "par_check"
    r = subprocess.run(["g++", "-std=c++17", "-O2", "-fopenmp", "-Wall", "-Werror", "-I" + CSRC, str(src), "-o",
                        str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    env = dict(os.environ, OMP_NUM_THREADS=str(threads))
    r = subprocess.run([str(exe)], capture_output=True, text=True, env=env, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "0", r.stdout + r.stderr
