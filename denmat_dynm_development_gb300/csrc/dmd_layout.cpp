// Host construction of the column-block pair layout (see dmd_layout.h).
#include "dmd_layout.h"

#include <algorithm>
#include <numeric>

namespace dmd {

bool build_pair_layout(int nk, int nb, const double* e_w, long long npair, const uint64_t* k1, const uint64_t* k2,
                       int pairs_per_item, int width, PairLayout& L) {
  // energy ranks
  std::vector<double> eb(nk);
  for (int k = 0; k < nk; ++k) {
    double s = 0;
    for (int b = 0; b < nb; ++b) s += e_w[(size_t)k * nb + b];
    eb[k] = s / nb;
  }
  L.inv.resize(nk);
  std::iota(L.inv.begin(), L.inv.end(), 0);
  std::stable_sort(L.inv.begin(), L.inv.end(), [&](int a, int b) { return eb[a] < eb[b]; });
  L.pos.assign(nk, 0);
  for (int r = 0; r < nk; ++r) L.pos[L.inv[r]] = r;
  // sort pairs by (column block, row, lane slot)
  std::vector<uint64_t> key(npair);
  std::vector<uint8_t> tr(npair, 0);
  std::vector<int32_t> prow(npair), pcol(npair);
  for (long long p = 0; p < npair; ++p) {
    if (k1[p] >= (uint64_t)nk || k2[p] >= (uint64_t)nk) return false;
    int r = L.pos[k1[p]], c = L.pos[k2[p]];
    if (k1[p] < k2[p] && r > c) {  // both directions: store with row <= column
      std::swap(r, c);
      tr[p] = 1;
    }
    prow[p] = r;
    pcol[p] = c;
    key[p] = ((uint64_t)(c / width) << 37) | ((uint64_t)r << 5) | (uint64_t)(c % width);  // nk < 2^31
  }
  std::vector<uint32_t> ord(npair);
  std::iota(ord.begin(), ord.end(), 0u);
  std::stable_sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return key[a] < key[b]; });
  L.src.resize(npair);
  L.slot_of.resize(npair);
  L.transposed.resize(npair);
  L.rb.clear();
  L.items.clear();
  // row blocks; a repeated (row, column) pair starts a new block so that slots stay unique
  long long q = 0;
  while (q < npair) {
    const uint32_t p = ord[q];
    const int row = prow[p];
    const int J = pcol[p] / width;
    RowBlock b;
    b.row = row;
    b.mask = 0;
    b.revmask = 0;
    b.pair0 = (uint32_t)q;
    long long e = q;
    while (e < npair) {
      const uint32_t pe = ord[e];
      const int c = pcol[pe];
      if (prow[pe] != row || c / width != J) break;
      const uint32_t bit = 1u << (c % width);
      if (b.mask & bit) break;  // duplicate pair: next block
      b.mask |= bit;
      if (k1[pe] < k2[pe]) b.revmask |= bit;
      ++e;
    }
    // slots in increasing lane order (the sort already orders by lane)
    for (long long i = q; i < e; ++i) {
      L.src[i] = ord[i];
      L.slot_of[i] = (uint8_t)(i - q);
      L.transposed[i] = tr[ord[i]];
    }
    L.rb.push_back(b);
    q = e;
  }
  // work items: runs of row blocks of one column block, about pairs_per_item pairs each
  size_t i = 0;
  while (i < L.rb.size()) {
    const int J = pcol[L.src[L.rb[i].pair0]] / width;
    WorkItem w;
    w.J = J;
    w.rb0 = (int32_t)i;
    long long np = 0;
    while (i < L.rb.size() && pcol[L.src[L.rb[i].pair0]] / width == J && np < pairs_per_item &&
           (int)(i - w.rb0) < kMaxRowBlocksPerItem) {
      np += __builtin_popcount(L.rb[i].mask);
      ++i;
    }
    w.rb1 = (int32_t)i;
    L.items.push_back(w);
  }
  return true;
}

}  // namespace dmd
