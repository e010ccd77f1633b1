// Host-side work partition of a chemistry box list across ranks (one rank per GPU).
//
// PeleLM balances its chemistry by cost on CPU builds: it chops the level's grids until there
// are at least chem_box_chop_threshold boxes per rank, never below 16 cells a side
// (Source/PeleLM.cpp:5699-5723), then assigns the boxes to ranks with a knapsack over each
// box's summed FuncCount of the previous advance (getFuncCountDM, Source/PeleLM.cpp:5530-5623;
// the assignment itself is AMReX's KnapSackProcessorMap). The cells are independent ODEs, so a
// shard needs no communication while it advances; only these weights cross ranks between steps.
//
// pgb_chop_boxes      halves the longest side of the largest box until the list is long enough
// pgb_partition_boxes longest-processing-time greedy, then move/swap refinement between the most
//                     and least loaded ranks while the largest load strictly drops
// The weights are the caller's per-box sums of FC from the previous advance (an FArrayBox sum in
// PeleLM, a tensor sum in Python), or cell counts before the first one.
#include <algorithm>
#include <cstdint>
#include <numeric>
#include <queue>
#include <vector>

#include "../../include/pelelm_gb300.h"

namespace pgb_host {
int set_err(const char* fmt, ...);
}
using pgb_host::set_err;

namespace {

long long cells_of(const pgb_box& b) {
  return (long long)(b.hi[0] - b.lo[0] + 1) * (b.hi[1] - b.lo[1] + 1) * (b.hi[2] - b.lo[2] + 1);
}

}  // namespace

extern "C" {

int pgb_chop_boxes(const pgb_box* in, int nin, int min_side, int target, pgb_box* out, int* parent, int cap) {
  if (nin < 0 || (nin > 0 && !in)) return set_err("chop_boxes: bad input list");
  if (min_side < 1) return set_err("chop_boxes: min_side must be >= 1");
  if (cap < nin || (cap > 0 && (!out || !parent))) return set_err("chop_boxes: output capacity %d < %d boxes", cap, nin);
  std::vector<pgb_box> boxes(in, in + nin);
  std::vector<int> par(nin);
  std::iota(par.begin(), par.end(), 0);
  for (int b = 0; b < nin; ++b)
    for (int d = 0; d < 3; ++d)
      if (in[b].hi[d] < in[b].lo[d]) return set_err("chop_boxes: box %d is empty in dim %d", b, d);
  // largest box first (ties: lowest index), split across its longest side if both halves keep
  // at least min_side cells there
  while ((int)boxes.size() < target && (int)boxes.size() < cap) {
    int best = -1, bd = 0;
    long long bc = 0;
    for (int b = 0; b < (int)boxes.size(); ++b) {
      int d = 0, len = 0;
      for (int k = 0; k < 3; ++k) {
        const int l = boxes[b].hi[k] - boxes[b].lo[k] + 1;
        if (l > len) { len = l; d = k; }
      }
      if (len < 2 * min_side) continue;
      const long long c = cells_of(boxes[b]);
      if (c > bc) { bc = c; best = b; bd = d; }
    }
    if (best < 0) break;
    pgb_box a = boxes[best], c = boxes[best];
    const int len = a.hi[bd] - a.lo[bd] + 1;
    a.hi[bd] = a.lo[bd] + len / 2 - 1;
    c.lo[bd] = a.hi[bd] + 1;
    boxes[best] = a;
    boxes.insert(boxes.begin() + best + 1, c);
    par.insert(par.begin() + best + 1, par[best]);
  }
  std::copy(boxes.begin(), boxes.end(), out);
  std::copy(par.begin(), par.end(), parent);
  return (int)boxes.size();
}

int pgb_partition_boxes(const double* weight, int nbox, int nranks, int* rank_of_box, double* load) {
  if (nbox < 0 || (nbox > 0 && (!weight || !rank_of_box))) return set_err("partition_boxes: bad arguments");
  if (nranks < 1) return set_err("partition_boxes: nranks must be >= 1");
  for (int b = 0; b < nbox; ++b)
    if (!(weight[b] >= 0.0)) return set_err("partition_boxes: weight of box %d is negative or NaN", b);
  std::vector<double> L(nranks, 0.0);
  // longest processing time first: heaviest box to the least loaded rank (ties: lowest rank)
  std::vector<int> order(nbox);
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](int a, int b) { return weight[a] > weight[b]; });
  using Item = std::pair<double, int>;
  std::priority_queue<Item, std::vector<Item>, std::greater<Item>> heap;
  for (int r = 0; r < nranks; ++r) heap.push({0.0, r});
  for (int b : order) {
    Item it = heap.top();
    heap.pop();
    rank_of_box[b] = it.second;
    it.first += weight[b];
    L[it.second] = it.first;
    heap.push(it);
  }
  // refinement: move one box, or swap two, between the most and the least loaded rank while
  // that strictly lowers the larger of their two loads
  for (int iter = 0; iter < 4 * nbox + 16 && nranks > 1; ++iter) {
    const int hi = (int)(std::max_element(L.begin(), L.end()) - L.begin());
    const int lo = (int)(std::min_element(L.begin(), L.end()) - L.begin());
    const double cur = L[hi];
    double best = cur;
    int ba = -1, bb = -1;
    std::vector<int> on_hi, on_lo;
    for (int b = 0; b < nbox; ++b) {
      if (rank_of_box[b] == hi) on_hi.push_back(b);
      else if (rank_of_box[b] == lo) on_lo.push_back(b);
    }
    for (int a : on_hi) {
      const double m = std::max(L[hi] - weight[a], L[lo] + weight[a]);
      if (m < best) { best = m; ba = a; bb = -1; }
      for (int b : on_lo) {
        if (!(weight[b] < weight[a])) continue;
        const double d = weight[a] - weight[b];
        const double s = std::max(L[hi] - d, L[lo] + d);
        if (s < best) { best = s; ba = a; bb = b; }
      }
    }
    if (ba < 0) break;
    rank_of_box[ba] = lo;
    L[hi] -= weight[ba];
    L[lo] += weight[ba];
    if (bb >= 0) {
      rank_of_box[bb] = hi;
      L[lo] -= weight[bb];
      L[hi] += weight[bb];
    }
  }
  if (load) {  // exact sums (the running totals above may have drifted in the last bits)
    std::fill(L.begin(), L.end(), 0.0);
    for (int b = 0; b < nbox; ++b) L[rank_of_box[b]] += weight[b];
    std::copy(L.begin(), L.end(), load);
  }
  return 0;
}

}  // extern "C"
