// Device layout of the k-pair operators for the column-block contraction kernels.
//
// k-points are ranked by their mean band energy (pos[k]); with the energy-window pair selection of
// the Lindblad initializer this turns the set of stored pairs into a band around the diagonal of
// the (pos[k1], pos[k2]) plane. Pairs are grouped by column block J = pos[k2] / W (W = 32 for nb = 2,
// 8 for nb = 4, where four lanes share a pair) and, inside a block, by row pos[k1]: a "row block"
// holds the pairs of one row whose columns fall in one column block, one per slot (slot s <-> column
// W J + s). A row block stores its P1 and P2 elements
// element-major ([element][slot]) so that a warp reads each element of all its pairs with one
// coalesced access. Work items are runs of row blocks of the same column block.
//
// A pair that carries both directions (k1 < k2, evolve_eph.cpp:101) may be stored transposed, as
// the pair (k2, k1) with P1' = conj(P2), P2' = conj(P1) -- the identity the reference itself uses
// for the k' side (evolve_eph.cpp:102-105). Every such pair is oriented so that its row precedes
// its column in energy order, which folds the band onto one side of the diagonal and fills the
// row blocks densely. Pairs without the reverse term keep their stored orientation.
#pragma once
#include <stdint.h>

#include <vector>

namespace dmd {

struct RowBlock {
  int32_t row;       // pos of the forward target k1
  uint32_t mask;     // slots holding a pair
  uint32_t revmask;  // slots whose pair also has the reverse (k' side) term: k1 < k2 as stored
  uint32_t pair0;    // index of the block's first pair in the permuted pair order
};

// row blocks per work item at most: the contraction kernel keeps one descriptor per lane
constexpr int kMaxRowBlocksPerItem = 32;

struct WorkItem {
  int32_t J;         // column block
  int32_t rb0, rb1;  // row blocks [rb0, rb1)
};

struct PairLayout {
  std::vector<int32_t> pos;       // k -> energy rank
  std::vector<int32_t> inv;       // energy rank -> k
  std::vector<RowBlock> rb;
  std::vector<WorkItem> items;
  std::vector<uint32_t> src;      // permuted pair slot -> source pair index
  std::vector<uint8_t> slot_of;   // permuted pair slot -> slot within its row block
  std::vector<uint8_t> transposed;  // permuted pair slot stored as (k2, k1) with (conj P2, conj P1)
};

// Builds the layout from the stored pairs. e_w is [nk][nb] (window energies), width the columns per
// column block (<= 32). Returns false on an out-of-range pair index.
bool build_pair_layout(int nk, int nb, const double* e_w, long long npair, const uint64_t* k1, const uint64_t* k2,
                       int pairs_per_item, int width, PairLayout& L);

}  // namespace dmd
