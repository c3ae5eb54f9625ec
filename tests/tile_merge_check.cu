// Host check of the tiled kernel's merge_skipped rule, built with nvcc and run
// on the CPU by tests/test_tile_merge.py.  For random tiles it compares two
// summaries:
//   - the full summary: the smallest key lower bound and its slot (the lowest
//     among equal bounds), that slot's key upper bound and neighbour field,
//     and the smallest bound of the other members without the winner's mutual
//     partner;
//   - the summary that merge_skipped builds from the parts of the members
//     other than slot a (tile_part's rule, restated below) and a's own key.
// The tiles have few distinct key values (many ties), neighbours inside and
// outside the tile, and planted mutual pairs.  Prints "ok <trials>".
#include <cmath>
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>

#include "fjg_cluster_tiled.cuh"

using namespace fjg;

namespace {

struct Slot {
  float klo, khi;
  int nn;
  bool pair;
};

int nnk_of(const Slot& s) { return (s.nn < 0 ? kNoNeighbour : s.nn) | (s.pair ? (int)kPairBit : 0); }

bool less_key(float k1, int s1, float k2, int s2) { return k1 < k2 || (k1 == k2 && s1 < s2); }

// tile_summary's definition over `members`
TileSum full(const std::vector<int>& members, const std::vector<Slot>& st) {
  const float inf = INFINITY;
  int x = -1;
  for (int u : members)
    if (x < 0 || less_key(st[u].klo, u, st[x].klo, x)) x = u;
  if (x < 0) return TileSum{inf, -1, inf, inf, kNoNeighbour, 0, 0, 0};
  const Slot& sx = st[x];
  const int p = (sx.pair && sx.nn >= 0 && st[sx.nn].pair && st[sx.nn].nn == x) ? sx.nn : -1;
  float mo = inf;
  for (int u : members)
    if (u != x && u != p) mo = std::fmin(mo, st[u].klo);
  return TileSum{sx.klo, x, sx.khi, mo, nnk_of(sx), 0, 0, 0};
}

// tile_part's definition over `members` other than `skip`
TilePart part(const std::vector<int>& members, int skip, const std::vector<Slot>& st) {
  const float inf = INFINITY;
  int x = -1;
  for (int u : members)
    if (u != skip && (x < 0 || less_key(st[u].klo, u, st[x].klo, x))) x = u;
  if (x < 0) return TilePart{inf, -1, inf, kNoNeighbour, inf};
  const Slot& sx = st[x];
  const int p = (sx.pair && sx.nn >= 0 && sx.nn != skip && st[sx.nn].pair && st[sx.nn].nn == x) ? sx.nn : -1;
  float mo = inf;
  for (int u : members)
    if (u != skip && u != x && u != p) mo = std::fmin(mo, st[u].klo);
  return TilePart{sx.klo, x, sx.khi, nnk_of(sx), mo};
}

bool same(const TileSum& a, const TileSum& b) {
  return std::memcmp(&a.m1, &b.m1, 4) == 0 && a.slot == b.slot && std::memcmp(&a.u1, &b.u1, 4) == 0 &&
         std::memcmp(&a.m2, &b.m2, 4) == 0 && a.nnk == b.nnk;
}

}  // namespace

int main() {
  std::mt19937_64 rng(20261204);
  const float keys[] = {0.5f, 1.0f, 1.5f, 2.0f, 2.5f};
  const int trials = 200000;
  for (int t = 0; t < trials; ++t) {
    const int n_slots = 4 + (int)(rng() % 14);
    std::vector<Slot> st(n_slots);
    for (auto& s : st) {
      s.klo = keys[rng() % 5];
      s.khi = (rng() % 2) ? s.klo : s.klo + 0.25f;
      s.nn = (int)(rng() % (n_slots + 1)) - 1;
      s.pair = (rng() % 10) < 7;
    }
    std::vector<int> members;
    for (int u = 0; u < n_slots; ++u)
      if (rng() % 3) members.push_back(u);
    if (members.empty()) members.push_back(0);
    const int a = members[rng() % members.size()];
    if (members.size() > 1 && rng() % 2) {  // plant a mutual pair with a
      int y = a;
      while (y == a) y = members[rng() % members.size()];
      st[a].nn = y;
      st[y].nn = a;
      st[a].pair = st[y].pair = true;
    }
    for (int u = 0; u < n_slots; ++u)
      if (st[u].nn == u) st[u].nn = -1;
    const TileSum ref = full(members, st);
    const TileSum got = merge_skipped(part(members, a, st), a, st[a].klo, st[a].khi, nnk_of(st[a]));
    if (!same(ref, got)) {
      std::printf("mismatch at trial %d: slot %d vs %d, m2 %g vs %g\n", t, ref.slot, got.slot, ref.m2, got.m2);
      return 1;
    }
  }
  std::printf("ok %d\n", trials);
  return 0;
}
