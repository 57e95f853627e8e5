"""The summation trees of device preprocessing (ennemi_gb300/csrc/egb_pwtree.h),
compiled with the host compiler: evaluated as the rescale kernels evaluate
them -- every leaf summed with eight accumulators, then the inner nodes one
height at a time -- they reproduce np.add.reduce of 1-D float64 arrays bit for
bit, and their structure is well formed (leaves tile [0, n) in order, every
inner node sits above its children, the root is last).
"""

import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

SIZES = [1, 2, 7, 8, 9, 15, 16, 17, 100, 127, 128, 129, 130, 136, 200, 255, 256, 257,
         1000, 1023, 1024, 1025, 4095, 8191, 8192, 8193, 20011, 65537, 180000]

HARNESS = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "egb_pwtree.h"

struct Node { int x, y; };
struct Tree { int32_t node0, nleaf, nnode, lvl0, nlvl; };

// one leaf of NumPy's pairwise_sum
static double leaf(const double* a, int len) {
  if (len < 8) {
    double r = 0.0;
    for (int i = 0; i < len; ++i) r += a[i];
    return r;
  }
  double r[8];
  for (int j = 0; j < 8; ++j) r[j] = a[j];
  int i = 8;
  for (; i < len - (len % 8); i += 8)
    for (int j = 0; j < 8; ++j) r[j] += a[i + j];
  double res = ((r[0] + r[1]) + (r[2] + r[3])) + ((r[4] + r[5]) + (r[6] + r[7]));
  for (; i < len; ++i) res += a[i];
  return res;
}

// stdin: n, then n doubles as raw bits (hex); stdout: the sum's bits, then
// "ok" if the tree is well formed
int main() {
  long long n;
  while (std::scanf("%lld", &n) == 1) {
    std::vector<double> a((size_t)n);
    for (auto& v : a) {
      unsigned long long b;
      if (std::scanf("%llx", &b) != 1) return 2;
      __builtin_memcpy(&v, &b, 8);
    }
    std::vector<Tree> trees;
    std::vector<Node> nodes;
    std::vector<int32_t> levels;
    const int t = egb::pw_build(n, trees, nodes, levels);
    const Tree& T = trees[(size_t)t];
    bool ok = T.nnode == (int)nodes.size() && (int)levels.size() == T.nlvl + 1 &&
              levels.back() == T.nnode;
    long long next = 0;  // leaves tile [0, n) in order, each at most 128 long
    for (int i = 0; i < T.nleaf; ++i) {
      ok = ok && nodes[(size_t)i].x == next && nodes[(size_t)i].y >= 1 && nodes[(size_t)i].y <= 128;
      next += nodes[(size_t)i].y;
    }
    ok = ok && next == n;
    std::vector<double> s((size_t)T.nnode);
    std::vector<int> height((size_t)T.nnode, 0);
    for (int i = 0; i < T.nleaf; ++i) s[(size_t)i] = leaf(a.data() + nodes[(size_t)i].x, nodes[(size_t)i].y);
    for (int h = 0; h < T.nlvl; ++h)
      for (int i = levels[(size_t)h]; i < levels[(size_t)h + 1]; ++i) {
        const Node c = nodes[(size_t)i];
        ok = ok && c.x < levels[(size_t)h] && c.y < levels[(size_t)h];  // children below
        ok = ok && std::max(height[(size_t)c.x], height[(size_t)c.y]) == h;
        height[(size_t)i] = h + 1;
        s[(size_t)i] = s[(size_t)c.x] + s[(size_t)c.y];
      }
    unsigned long long out;
    __builtin_memcpy(&out, &s[(size_t)T.nnode - 1], 8);
    std::printf("%llx %s\n", out, ok ? "ok" : "bad");
  }
  return 0;
}
"""


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    d = tmp_path_factory.mktemp("pwtree")
    src = d / "pw.cc"
    src.write_text(HARNESS)
    exe = d / "pw"
    subprocess.check_call([cxx, "-std=c++17", "-O2", "-ffp-contract=off",
                           "-I", os.path.join(ROOT, "ennemi_gb300", "csrc"), str(src), "-o", str(exe)])
    return exe


def test_trees_sum_like_numpy(harness):
    rng = np.random.default_rng(41)
    arrays = []
    for n in SIZES:
        for scale in (1.0, 1e-3, 1e6):
            arrays.append(rng.standard_normal(n) * scale + rng.uniform(-3, 3) * scale)
    text = "".join(f"{len(a)}\n" + " ".join(f"{b:x}" for b in a.view(np.uint64)) + "\n" for a in arrays)
    out = subprocess.run([str(harness)], input=text, capture_output=True, text=True, check=True)
    lines = out.stdout.split("\n")
    for a, line in zip(arrays, lines):
        bits, ok = line.split()
        assert ok == "ok", len(a)
        want = np.array([np.add.reduce(a)]).view(np.uint64)[0]
        assert int(bits, 16) == int(want), len(a)
