"""The dynamic shared-memory limit cache (csrc/smem_limit.h) only ever raises a
kernel's limit, per device, under one lock.

The red-black HBS factorisation compresses one level's operators on worker
threads, each at its own tree level, so one kernel is launched concurrently at
several shared-memory sizes (omsdirectsolveHBS.py:436-483 _build_level runs
three compressions per kept node).  A limit that a thread could lower between
another thread's set and launch made that launch fail with 'invalid argument'.
This test compiles the header with a fake setter on the host: no GPU."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "sslablu_gb300", "csrc")

PROGRAM = r"""
#include "smem_limit.h"
#include <atomic>
#include <cstdio>
#include <thread>
#include <vector>

int main() {
  slu::SmemLimit c;
  int k1 = 0, k2 = 0;
  const void* a = &k1;
  const void* b = &k2;
  std::vector<std::size_t> sets;
  auto rec = [&](std::size_t v) { sets.push_back(v); return 0; };
  // at or below the default: no call
  if (c.raise(0, a, 48 * 1024, rec) != 0 || !sets.empty()) return 1;
  // raises, then never lowers
  c.raise(0, a, 100000, rec);
  c.raise(0, a, 60000, rec);
  c.raise(0, a, 100000, rec);
  c.raise(0, a, 150000, rec);
  if (sets.size() != 2 || sets[0] != 100000 || sets[1] != 150000) return 2;
  if (c.current(0, a) != 150000) return 3;
  // per kernel and per device
  c.raise(0, b, 70000, rec);
  c.raise(1, a, 70000, rec);
  if (sets.size() != 4 || c.current(1, a) != 70000 || c.current(0, b) != 70000) return 4;
  // a failed set is not remembered
  auto fail = [&](std::size_t) { return 7; };
  if (c.raise(2, a, 90000, fail) != 7 || c.current(2, a) != 0) return 5;
  // many threads at mixed sizes: the value seen by the setter never drops
  slu::SmemLimit d;
  std::atomic<std::size_t> last{0};
  std::atomic<int> drops{0};
  auto mono = [&](std::size_t v) {
    std::size_t prev = last.exchange(v);
    if (v < prev) drops++;
    return 0;
  };
  std::vector<std::thread> th;
  for (int t = 0; t < 12; ++t)
    th.emplace_back([&, t] {
      for (int i = 0; i < 2000; ++i) {
        std::size_t want = 50000 + (std::size_t)((i * 7919 + t * 104729) % 170000);
        d.raise(0, a, want, mono);
        if (d.current(0, a) < want) drops++;
      }
    });
  for (auto& x : th) x.join();
  if (drops.load() != 0) return 6;
  std::printf("ok %zu\n", d.current(0, a));
  return 0;
}
"""


def test_smem_limit_only_grows():
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "t.cpp")
        exe = os.path.join(tmp, "t")
        with open(src, "w") as f:
            f.write(PROGRAM)
        r = subprocess.run([gxx, "-std=c++17", "-O1", "-pthread", "-I", CSRC, src, "-o", exe],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
        assert r.returncode == 0, "smem limit check failed with code %d" % r.returncode
        assert r.stdout.startswith("ok")
