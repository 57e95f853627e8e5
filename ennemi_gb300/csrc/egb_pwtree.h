// egb_pwtree.h -- NumPy's pairwise summation order as a tree (host code only,
// no CUDA: the library's planner and a compiled test share it).
//
// NumPy sums a contiguous 1-D float64 array -- np.add.reduce, mean() and
// std() -- by pairwise_sum (numpy/_core/src/umath/loops_utils.h.src): n <= 128
// values are summed directly (fewer than 8 in order from 0.0, else eight
// running sums over strides of 8, combined ((r0+r1)+(r2+r3))+((r4+r5)+(r6+r7)),
// then the last n % 8 in order), larger n is split at n2 = n / 2 rounded down
// to a multiple of 8 and the two halves' sums added.
//
// pw_build stores that recursion for one n: the leaves first, in order, as
// (offset, length), then the inner nodes as (left, right) child indices,
// ordered by height so that the nodes of one height depend only on lower
// ones; levels gets the first node index of each height 1 .. H and then the
// node count.  The root is the last node.
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

namespace egb {

// Node: an aggregate of two ints (x, y); Tree: has int32 node0, nleaf,
// nnode, lvl0, nlvl.  Appends to the three vectors; returns the tree's index.
template <class Node, class Tree>
int32_t pw_build(int64_t n, std::vector<Tree>& trees, std::vector<Node>& nodes,
                 std::vector<int32_t>& levels) {
  struct Ref { bool leaf; int32_t i; };
  struct Inner { Ref l, r; int h; };
  std::vector<Node> leaves;
  std::vector<Inner> inner;
  // explicit recursion (depth about log2(n / 64))
  struct Frame { int64_t off, m; int stage; Ref l; int hl; };
  std::vector<Frame> stack{{0, n, 0, {true, 0}, 0}};
  Ref ret{true, 0};
  int ret_h = 0;
  while (!stack.empty()) {
    Frame& f = stack.back();
    if (f.m <= 128) {
      leaves.push_back(Node{(int)f.off, (int)f.m});
      ret = {true, (int32_t)leaves.size() - 1};
      ret_h = 0;
      stack.pop_back();
      continue;
    }
    int64_t m2 = f.m / 2;
    m2 -= m2 % 8;
    if (f.stage == 0) {
      f.stage = 1;
      stack.push_back({f.off, m2, 0, {true, 0}, 0});
    } else if (f.stage == 1) {
      f.stage = 2;
      f.l = ret;
      f.hl = ret_h;
      const int64_t off = f.off + m2, m = f.m - m2;
      stack.push_back({off, m, 0, {true, 0}, 0});  // f is not used after this
    } else {
      const int h = 1 + std::max(f.hl, ret_h);
      inner.push_back({f.l, ret, h});
      ret = {false, (int32_t)inner.size() - 1};
      ret_h = h;
      stack.pop_back();
    }
  }
  std::vector<int32_t> order(inner.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int32_t)i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int32_t a, int32_t b) { return inner[(size_t)a].h < inner[(size_t)b].h; });
  const int32_t L = (int32_t)leaves.size();
  std::vector<int32_t> pos(inner.size());
  for (size_t k = 0; k < order.size(); ++k) pos[(size_t)order[k]] = L + (int32_t)k;
  auto idx = [&](Ref r) { return r.leaf ? r.i : pos[(size_t)r.i]; };
  Tree T{};
  T.node0 = (int32_t)nodes.size();
  T.nleaf = L;
  T.nnode = L + (int32_t)inner.size();
  T.lvl0 = (int32_t)levels.size();
  nodes.insert(nodes.end(), leaves.begin(), leaves.end());
  int H = 0;
  for (size_t k = 0; k < order.size(); ++k) {
    const Inner& in = inner[(size_t)order[k]];
    nodes.push_back(Node{idx(in.l), idx(in.r)});
    if (in.h > H) {  // first node of height in.h
      levels.push_back(L + (int32_t)k);
      H = in.h;
    }
  }
  T.nlvl = H;
  levels.push_back(T.nnode);
  trees.push_back(T);
  return (int32_t)trees.size() - 1;
}

}  // namespace egb
