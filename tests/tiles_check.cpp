// Host check of the mixed mode's tile plan (rocflu_gb300/csrc/tiles.h) on an
// n^3 hex box: cells in Morton order, vertex-neighbour stencils (26 members
// inside), six face entries per cell in the order -x +x -y +y -z +z with the
// box faces as boundary entries.  Built and run by tests/test_tiles_cpu.py.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <random>
#include <vector>

#include "tiles.h"

namespace {

int fails = 0;
#define CHECK(c)                                                  \
  do {                                                            \
    if (!(c)) {                                                   \
      std::printf("FAIL %s:%d %s\n", __FILE__, __LINE__, #c);     \
      ++fails;                                                    \
    }                                                             \
  } while (0)

unsigned spread3(unsigned x) {
  unsigned r = 0;
  for (int b = 0; b < 10; ++b) r |= ((x >> b) & 1u) << (3 * b);
  return r;
}

struct Mesh {
  int nc = 0;
  std::vector<int> cfOff, cfEnt, stOff, stIdx, fc1, fc2;
};

// n a power of two: Morton index of (i, j, k) = interleaved bits.  perm maps
// the Morton index to the stored cell id (identity: Morton order).
Mesh hexBox(int n, const std::vector<int> &perm) {
  Mesh m;
  m.nc = n * n * n;
  auto at = [&](int i, int j, int k) { return perm[spread3(i) | spread3(j) << 1 | spread3(k) << 2]; };
  std::vector<int> ii(m.nc), jj(m.nc), kk(m.nc);
  for (int k = 0; k < n; ++k)
    for (int j = 0; j < n; ++j)
      for (int i = 0; i < n; ++i) {
        const int c = at(i, j, k);
        ii[c] = i; jj[c] = j; kk[c] = k;
      }
  // interior faces: one per (cell, +direction) pair inside the box
  const int dirs[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  std::vector<std::vector<int>> entDir(m.nc, std::vector<int>(6, -1));
  int nb = 0;
  for (int c = 0; c < m.nc; ++c)
    for (int d = 0; d < 3; ++d) {
      const int i2 = ii[c] + dirs[d][0], j2 = jj[c] + dirs[d][1], k2 = kk[c] + dirs[d][2];
      if (i2 < n && j2 < n && k2 < n) {
        const int c2 = at(i2, j2, k2), f = (int)m.fc1.size();
        m.fc1.push_back(c);
        m.fc2.push_back(c2);
        entDir[c][2 * d + 1] = 2 * f;       // c sees the face as its first side
        entDir[c2][2 * d] = 2 * f + 1;      // c2 as the second
      }
    }
  m.cfOff.assign(m.nc + 1, 0);
  for (int c = 0; c < m.nc; ++c) {
    for (int s = 0; s < 6; ++s) m.cfEnt.push_back(entDir[c][s] >= 0 ? entDir[c][s] : -(++nb));
    m.cfOff[c + 1] = (int)m.cfEnt.size();
  }
  m.stOff.assign(m.nc + 1, 0);
  for (int c = 0; c < m.nc; ++c) {
    std::vector<int> st;
    for (int dk = -1; dk <= 1; ++dk)
      for (int dj = -1; dj <= 1; ++dj)
        for (int di = -1; di <= 1; ++di) {
          const int i2 = ii[c] + di, j2 = jj[c] + dj, k2 = kk[c] + dk;
          if ((di || dj || dk) && i2 >= 0 && j2 >= 0 && k2 >= 0 && i2 < n && j2 < n && k2 < n)
            st.push_back(at(i2, j2, k2));
        }
    m.stIdx.insert(m.stIdx.end(), st.begin(), st.end());
    m.stOff[c + 1] = (int)m.stIdx.size();
  }
  return m;
}

// Every local id resolves to the cell it stands for; the halo lists hold each
// halo cell once and -1 elsewhere; aligned plans keep the low three bits.
void checkPlan(const Mesh &m, const rflu::TilePlan &p, int tile) {
  const int nTiles = (m.nc + tile - 1) / tile;
  CHECK((int)p.haloOff.size() == nTiles + 1);
  for (int t = 0; t < nTiles; ++t) {
    const int b0 = t * tile, b1 = std::min(m.nc, b0 + tile), hb = p.haloOff[t];
    CHECK(p.haloOff[t + 1] - hb + tile <= p.maxRecs);
    auto cellOf = [&](int l) { return l < tile ? b0 + l : p.haloIdx[hb + l - tile]; };
    std::vector<int> seen;
    // every list starts on a 16-byte boundary; compact lists are padded
    // with at most three unused slots at their end
    CHECK(hb % 4 == 0);
    for (int h = hb; h < p.haloOff[t + 1]; ++h) {
      const int j = p.haloIdx[h];
      if (j < 0) {
        CHECK(p.aligned || h >= p.haloOff[t + 1] - 3);
        continue;
      }
      CHECK(j < b0 || j >= b1);
      seen.push_back(j);
      if (p.aligned) CHECK(((tile + h - hb) & 7) == (j & 7));
    }
    std::sort(seen.begin(), seen.end());
    CHECK(std::adjacent_find(seen.begin(), seen.end()) == seen.end());
    for (int i = b0; i < b1; ++i) {
      for (int s = m.stOff[i]; s < m.stOff[i + 1]; ++s) CHECK(cellOf(p.stLoc[s]) == m.stIdx[s]);
      for (int e = m.cfOff[i]; e < m.cfOff[i + 1]; ++e) {
        const int code = m.cfEnt[e];
        if (code < 0) {
          CHECK(p.entLoc[e] == -1);
        } else {
          const int f = code >> 1, nb = (code & 1) ? m.fc1[f] : m.fc2[f];
          CHECK(cellOf(p.entLoc[e]) == nb);
        }
      }
    }
  }
}

// 16-byte shared-memory wavefronts of the stencil loop (8 lanes of 4 per
// phase, the two halves of each 32-byte record swizzled by bit 2 of its
// local id), over ideal: 1 means no bank conflicts.
double stencilWavefronts(const Mesh &m, const rflu::TilePlan &p, int tile) {
  long long wf = 0, ideal = 0;
  for (int w0 = 0; w0 + 32 <= m.nc; w0 += 32) {
    int kmax = 0;
    for (int c = w0; c < w0 + 32; ++c) kmax = std::max(kmax, m.stOff[c + 1] - m.stOff[c]);
    for (int k = 0; k < kmax; ++k)
      for (int half = 0; half < 2; ++half)
        for (int ph = 0; ph < 4; ++ph) {
          std::vector<std::vector<int>> grp(8);
          bool any = false;
          for (int lane = 8 * ph; lane < 8 * ph + 8; ++lane) {
            const int c = w0 + lane;
            if (k >= m.stOff[c + 1] - m.stOff[c]) continue;
            const int l = p.stLoc[m.stOff[c] + k];
            int o = 8 * l + (l & 4);
            if (half) o ^= 4;
            const int unit = o / 4;
            auto &g = grp[unit & 7];
            if (std::find(g.begin(), g.end(), unit) == g.end()) g.push_back(unit);
            any = true;
          }
          if (!any) continue;
          size_t mx = 0;
          for (auto &g : grp) mx = std::max(mx, g.size());
          wf += (long long)mx;
          ++ideal;
        }
  }
  (void)tile;
  return (double)wf / (double)ideal;
}

}  // namespace

int main() {
  const int n = 16, tile = 256;
  std::vector<int> ident(n * n * n);
  std::iota(ident.begin(), ident.end(), 0);
  const Mesh morton = hexBox(n, ident);
  auto roomy = [](int, int, bool) { return (size_t)3; };  // shared memory never binds
  rflu::TilePlan pa, pc;
  CHECK(rflu::planTiles(morton.nc, tile, morton.cfOff, morton.cfEnt, morton.stOff, morton.stIdx, morton.fc1,
                        morton.fc2, roomy, pa));
  CHECK(pa.aligned);
  checkPlan(morton, pa, tile);
  // the same mesh when larger buffers would cost occupancy: compact slots
  auto tight = [](int recs, int, bool) { return (size_t)(100000 / recs); };
  CHECK(rflu::planTiles(morton.nc, tile, morton.cfOff, morton.cfEnt, morton.stOff, morton.stIdx, morton.fc1,
                        morton.fc2, tight, pc));
  checkPlan(morton, pc, tile);
  CHECK(pc.maxRecs <= pa.maxRecs);
  if (pc.maxRecs < pa.maxRecs) CHECK(!pc.aligned);
  const double wa = stencilWavefronts(morton, pa, tile), wc = stencilWavefronts(morton, pc, tile);
  CHECK(wa < 1.2);  // a third of a 16^3 box lies on its boundary, where stencils are shorter
  CHECK(wa < wc);
  // a shuffled cell order: no structure to align, every id still resolves
  std::vector<int> perm(ident);
  std::mt19937 rng(3);
  std::shuffle(perm.begin(), perm.end(), rng);
  const Mesh shuffled = hexBox(n, perm);
  rflu::TilePlan ps;
  CHECK(rflu::planTiles(shuffled.nc, tile, shuffled.cfOff, shuffled.cfEnt, shuffled.stOff, shuffled.stIdx,
                        shuffled.fc1, shuffled.fc2, tight, ps));
  checkPlan(shuffled, ps, tile);
  std::printf("aligned %d maxRecs %d wavefronts %.3f | compact %d maxRecs %d wavefronts %.3f | shuffled aligned %d maxRecs %d\n",
              (int)pa.aligned, pa.maxRecs, wa, (int)pc.aligned, pc.maxRecs, wc, (int)ps.aligned, ps.maxRecs);
  if (fails) {
    std::printf("%d checks failed\n", fails);
    return 1;
  }
  std::printf("ok\n");
  return 0;
}
