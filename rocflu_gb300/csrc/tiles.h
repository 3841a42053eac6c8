// Host-side plan of the mixed mode's tiles (plain C++, no CUDA): cells in
// tiles of `tile` consecutive (Morton-ordered) ids, each tile with the halo
// of outside cells its stencils and interior faces reach, and every stencil
// member and face neighbour addressed by a 16-bit local id into the tile's
// staged records (own cells 0..tile-1, halo slots after).
#pragma once
#include <algorithm>
#include <cstddef>
#include <vector>

namespace rflu {

struct TilePlan {
  std::vector<int> haloOff, haloIdx;   // CSR over tiles of halo cell ids by slot (-1: unused slot)
  std::vector<unsigned short> stLoc;   // stencil members as local ids (CSR of the stencil)
  std::vector<int> entLoc;             // neighbour local id per cell-face entry (-1: boundary entry)
  int maxRecs = 0;                     // staged records of the largest tile (own + halo slots)
  int maxTileSt = 0;                   // stencil members of the largest tile
  bool aligned = false;                // bank-aligned halo slots taken
};

// cfOff/cfEnt: per-cell face entries (code >= 0: interior face code >> 1 seen
// from side code & 1; < 0: boundary face); stOff/stIdx: stencil CSR; fc1/fc2:
// the two cells of each interior face.  ctasPerSm(recs, maxTileSt, venkat)
// gives the CTAs per SM that shared memory allows for tile buffers of that
// many records (with the Venkatakrishnan face-offset cache or not).
//
// Halo slots.  Compact: the halo cells, sorted, after the tile's own cells.
// Bank-aligned: a halo cell j takes slot 8 r + (j & 7), r counting the halo
// cells of its residue, so every staged record's local id keeps the low
// three bits of its cell id (own cells too when tile is a multiple of 8),
// and unused slots hold -1.  On a Morton-ordered structured mesh the k-th
// stencil members (and k-th face neighbours) of 8 consecutive cells then
// differ in those bits, and with the record swizzle their 16-byte loads hit
// 8 different shared-memory bank groups.  The aligned slots are taken
// unless their larger buffers would fit fewer CTAs per SM (unstructured
// meshes, whose residues are uneven).  Either way every tile's list holds a
// multiple of 4 slots (unused ones -1), so that each starts on a 16-byte
// boundary and the kernels copy it as whole 16-byte words.  Returns false
// when a tile would need more than 65535 records (the mesh then stays
// untiled).
template <class CtasPerSm>
inline bool planTiles(int nc, int tile, const std::vector<int> &cfOff, const std::vector<int> &cfEnt,
                      const std::vector<int> &stOff, const std::vector<int> &stIdx, const std::vector<int> &fc1,
                      const std::vector<int> &fc2, CtasPerSm ctasPerSm, TilePlan &p) {
  const int nTiles = (nc + tile - 1) / tile;
  p.haloOff.assign(nTiles + 1, 0);
  p.haloIdx.clear();
  p.stLoc.assign(stIdx.size(), 0);
  p.entLoc.assign(cfEnt.size(), -1);
  std::vector<int> mark(nc, -1), slot(nc, -1);
  auto other = [&](int e) {  // neighbour of a cell's interior face entry
    const int f = cfEnt[e] >> 1;
    return (cfEnt[e] & 1) ? fc1[f] : fc2[f];
  };
  // pass 1: each tile's halo (sorted ids of the cells outside the tile that
  // its stencils and interior faces reach)
  std::vector<std::vector<int>> halos(nTiles);
  for (int t = 0; t < nTiles; ++t) {
    const int b0 = t * tile, b1 = std::min(nc, b0 + tile);
    std::vector<int> &halo = halos[t];
    auto visit = [&](int j) {
      if ((j < b0 || j >= b1) && mark[j] != t) {
        mark[j] = t;
        halo.push_back(j);
      }
    };
    for (int i = b0; i < b1; ++i) {
      for (int s = stOff[i]; s < stOff[i + 1]; ++s) visit(stIdx[s]);
      for (int e = cfOff[i]; e < cfOff[i + 1]; ++e)
        if (cfEnt[e] >= 0) visit(other(e));
    }
    std::sort(halo.begin(), halo.end());
  }
  p.maxTileSt = 0;
  for (int t = 0; t < nTiles; ++t) {
    const int b0 = t * tile, b1 = std::min(nc, b0 + tile);
    p.maxTileSt = std::max(p.maxTileSt, stOff[b1] - stOff[b0]);
  }
  int compactRecs = 0, alignedRecs = 0;
  for (int t = 0; t < nTiles; ++t) {
    int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int j : halos[t]) cnt[j & 7]++;
    compactRecs = std::max(compactRecs, tile + ((int)halos[t].size() + 3) / 4 * 4);
    alignedRecs = std::max(alignedRecs, tile + 8 * *std::max_element(cnt, cnt + 8));
  }
  p.aligned = tile % 8 == 0 && alignedRecs <= 65535 &&
              ctasPerSm(alignedRecs, p.maxTileSt, false) >= ctasPerSm(compactRecs, p.maxTileSt, false) &&
              ctasPerSm(alignedRecs, p.maxTileSt, true) >= ctasPerSm(compactRecs, p.maxTileSt, true);
  p.maxRecs = p.aligned ? alignedRecs : compactRecs;
  if (p.maxRecs > 65535) return false;
  // pass 2: slots, local ids of stencil members and face neighbours, and the
  // slot-ordered halo lists
  for (int t = 0; t < nTiles; ++t) {
    const int b0 = t * tile, b1 = std::min(nc, b0 + tile);
    const std::vector<int> &halo = halos[t];
    int rows = 0;
    if (p.aligned) {
      int cnt[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      for (int j : halo) slot[j] = 8 * cnt[j & 7]++ + (j & 7);
      rows = *std::max_element(cnt, cnt + 8);
    } else {
      for (size_t k = 0; k < halo.size(); ++k) slot[halo[k]] = (int)k;
    }
    auto local = [&](int j) {
      if (j >= b0 && j < b1) return j - b0;
      return tile + slot[j];
    };
    for (int i = b0; i < b1; ++i) {
      for (int s = stOff[i]; s < stOff[i + 1]; ++s) p.stLoc[s] = (unsigned short)local(stIdx[s]);
      for (int e = cfOff[i]; e < cfOff[i + 1]; ++e)
        if (cfEnt[e] >= 0) p.entLoc[e] = local(other(e));
    }
    const size_t h0 = p.haloIdx.size();
    p.haloIdx.resize(h0 + (p.aligned ? 8 * (size_t)rows : (halo.size() + 3) / 4 * 4), -1);
    for (int j : halo) p.haloIdx[h0 + slot[j]] = j;
    p.haloOff[t + 1] = (int)p.haloIdx.size();
  }
  return true;
}

}  // namespace rflu
