// Clustering of large events (more than 4096 particles): one CTA per event,
// per-slot state in a global workspace (two 16 B records per slot, read with
// one gather each), the tile lists' ranges and the tile summaries in shared
// memory, nearest neighbours restricted to a 3x3 window of rapidity-azimuth
// tiles.  (The reference's grid backend, grid.cu:55-549,
// also tiles the plane with cells of side >= R and compares adjacent cells;
// it keeps per-cell pair minima, this kernel a per-slot neighbour table.)
//
// Tiles.  Rapidity is tiled over the event's range (clamped to [-15, 15]; a
// particle outside goes to the edge tile, which keeps the tile index monotone
// in rapidity), azimuth over [0, 2pi) with wrap-around.  Both sides are at
// least R (1 + 1e-4) + 1e-5, so two pseudojets closer than that lie in the
// same or in adjacent tiles; tile indices come from the exact FP64
// coordinates.  Slots never move (the new jet of a merge takes the slot
// a = min(c, j)), so the label of a slot (the lowest input index among its
// constituents) is the slot index itself.
//
// Why windows give the same winner as the all-pairs rule.  Let nn'(s) be the
// nearest neighbour of s within its window, key'(s) its key.  If the global
// nearest neighbour of s lies outside the window, every other pseudojet is at
// dR > R (1 + 1e-4) from s, so every pair distance of s exceeds the smaller
// of the two weights (also after rounding).  Then (i) if s wins the all-pairs
// argmin its key is the beam distance w_s (a pair key w_t dR^2/R^2 would
// exceed w_t >= key(t)), and every window candidate u has w_u >= w_s
// (otherwise key(u) <= w_u < w_s), so key'(s) = w_s as well; (ii) any other
// such s has key'(s) = w_s >= key(s), or key'(s) = w_u dR^2/R^2 > w_u >=
// key(u) for its window neighbour u, so it cannot undercut the winner.
// Pseudojets whose nearest neighbour is inside the window have identical
// keys in both rules.  Hence, with the same (key, label) order, the windowed
// argmin selects the same pseudojet, kind and partner as the all-pairs rule
// at every step.  Each candidate set must be exactly the window, so that a
// change of one pseudojet is seen by every slot whose neighbour it can be.
//
// Tile lists.  Per tile, a list of member slots with S.slack free entries
// after the live ones.  Removal writes a tombstone (-1) in place; a new jet
// that changes tile is appended.  The lists are rebuilt (tombstones squeezed
// out, every slack entry set to -1) every S.slack steps; at most one entry is
// appended per step.  The slack is what the list area spares per tile
// (kListSlack entries per possible tile, spread over the tiles in use), at
// most kTileSlackMax.
//
// The update runs on thread 0 in S3 while the other warps scan windows for
// the step's targets and the new jet's window, with no barrier or fence
// between them.  Its stores, and
// what a concurrent reader of the same words can observe (32-bit words, so
// each load returns the old or the new value, never a mix):
//   (1) members[start[tile b] + pos b] = -1: the reader sees b or -1;
//   (2) when a changes tile, members[start[old tile a] + pos a] = -1: a or -1;
//   (3) members[start[ta] + p] = a with p = count[ta], then count[ta] = p + 1:
//       a reader holding the old count never reaches entry p; one holding the
//       new count reads entry p as a or as its previous word, and that word
//       is -1 -- entry p lies past every count this tile has had since the
//       last rebuild (counts only grow between rebuilds, by one per append),
//       so nothing has written it since the rebuild set it to -1;
//   (4) pos[a], tile[a], alive[b] and the referrer counts of a and of one
//       dropped neighbour: no S3 reader uses them for a, b or as an index.
// Every outcome is a, b or -1, and every reader skips -1 and the merged slots
// c and j by name ({a, b} = {c, j}); the new jet a enters the targets'
// searches explicitly (`extra`), not through the lists.  So the scans find
// the same candidates whichever words they see.  Lengths are read once and
// clamped to the list capacity, which the slack bounds as above.  The
// barrier B3 then orders the completed update before the next readers.
//
// Per step (T = 256 threads, 8 warps):
//   S1  argmin over the tile summaries (smallest klo, its slot and khi,
//       second smallest klo), certified as in the small-event kernel,
//       otherwise an exact argmin over the contenders.                    B1
//   S2  warps 0-2 merge or promote (the new jet's kinematics and tile);
//       warps 3-7 find the slots whose neighbour was c or j (in the windows
//       of c's and j's tiles) and scan the first 32 of them.               B2
//   S3  thread 0 updates the tile lists; the warps finish the targets'
//       neighbours, adding the new jet when it lies in their window, and
//       then compare every slot of the new jet's window with it, taking the
//       window's list positions in chunks of 32 (targets, flagged in S2, are
//       left to their own searches).                                      B3
//       (targets beyond the listed ones: a second pass, then a barrier)
//   S3c warp 0 resolves the new jet's neighbour while warp 1 summarises the
//       new jet's tile without it; warp 0 then merges the new jet's key in
//       (merge_skipped).  The other warps re-summarise the other changed
//       tiles (a winner there whose neighbour is the new jet may read the
//       new jet's fields mid-update: they only decide whether the new jet is
//       left out of that tile's second bound, and it is no member there). B4
#pragma once

#include "fjg_cluster.cuh"

namespace fjg {

constexpr int kTiledT = 256;
constexpr int kListSlack = 64;      // spare list entries per possible tile
// rebuild interval bound (steps): above what the spare area allows for the
// event sizes of interest (~870 steps at 40k particles), so that the area, not
// this bound, sets how rarely the lists are rebuilt (1024 against 256: pile-up
// batch +4 %, same-box A/B)
constexpr int kTileSlackMax = 1024;
constexpr int kMaxTiles = 4096;
// Tiles of one event in use, at most: their list ranges and key summaries live
// in shared memory (40 KB), so every phase reads them there and not through
// an L2 round trip.  Events that would want more get coarser tiles (still
// correct, see above): ~300 tiles at R = 0.4 over |y| < 4.
constexpr int kSmemTiles = 1024;
constexpr double kTileMembers = 32.0;  // particles per tile the tile side aims at (at least)
constexpr int kMaxWindowTiles = 9;
constexpr int kTiledTargets = 32;                // targets per step scanned during the merge
constexpr int kMaxListed = 4 * kTiledTargets;  // targets recorded in S2
constexpr int kMaxDirty = 64;
constexpr int kLargeWsBytesPerParticle = 96;  // bound of large_ws_bytes(N) / N for N > 2048

// Summary of one tile: the smallest key lower bound among its members, the
// member holding it (lowest slot among equal bounds) with its key upper
// bound and neighbour field (neighbour, kind in the top bit), and the second
// smallest lower bound without that member's mutual partner (see Cand).
struct alignas(16) TileSum {
  float m1;
  int slot;
  float u1;
  float m2;
  int nnk;
  int pad0, pad1, pad2;
};

// Summary parts of a tile's members other than one slot (tile_part).
struct TilePart {
  float m1;
  int x;
  float u1;
  int nnk;
  float mo;
};

constexpr int kNoNeighbour = 0x7fffffff;    // neighbour field without a neighbour
constexpr unsigned kPairBit = 0x80000000u;  // kind bit of the neighbour field: pair, not beam

// Partial argmin of the keys for the certificate.  m2 is the smallest lower
// bound among the other candidates, leaving out the best one's mutual
// partner: two slots that are each other's neighbour with pair keys hold the
// same exact key (the same FP64 expression of the same pair), and whichever
// of them wins, the step merges that pair, so their tie needs no FP64
// resolution.
struct Cand {
  float m1;  // smallest key lower bound
  int slot;  // its slot (the lowest among equal bounds), -1 if none
  float u1;  // its key upper bound
  int nnk;   // its neighbour field
  float m2;  // smallest lower bound of the others, without the mutual partner
};

__device__ __forceinline__ Cand cand_empty() {
  return Cand{__int_as_float(0x7f800000), -1, __int_as_float(0x7f800000), kNoNeighbour, __int_as_float(0x7f800000)};
}

__device__ __forceinline__ bool cand_partners(int slot_x, int nnk_x, int slot_y, int nnk_y) {
  return slot_x >= 0 && slot_y >= 0 && nnk_x == (int)((unsigned)slot_y | kPairBit) &&
         nnk_y == (int)((unsigned)slot_x | kPairBit);
}

// x <- the combination of partials x and y.
__device__ __forceinline__ void cand_merge(Cand& x, const Cand& y) {
  if (y.m1 < x.m1 || (y.m1 == x.m1 && (unsigned)y.slot < (unsigned)x.slot)) {
    const float cx = cand_partners(x.slot, x.nnk, y.slot, y.nnk) ? x.m2 : x.m1;
    x = Cand{y.m1, y.slot, y.u1, y.nnk, fminf(y.m2, cx)};
  } else {
    x.m2 = fminf(x.m2, cand_partners(y.slot, y.nnk, x.slot, x.nnk) ? y.m2 : y.m1);
  }
}

// Combination over a warp (every lane receives it).
__device__ __forceinline__ Cand cand_warp(const Cand& c) {
  const int lane = threadIdx.x & 31;
  const unsigned mb = __reduce_min_sync(kFull, __float_as_uint(c.m1));
  const bool at_min = __float_as_uint(c.m1) == mb && c.slot >= 0;
  const unsigned sb = __reduce_min_sync(kFull, at_min ? (unsigned)c.slot : 0xffffffffu);
  const unsigned ball = __ballot_sync(kFull, at_min && (unsigned)c.slot == sb);
  const int src = ball ? __ffs(ball) - 1 : 0;
  Cand r;
  r.m1 = __uint_as_float(mb);
  r.slot = ball ? (int)sb : -1;
  r.u1 = __shfl_sync(kFull, c.u1, src);
  r.nnk = __shfl_sync(kFull, c.nnk, src);
  const float contrib = (ball && lane == src) ? c.m2 : (cand_partners(c.slot, c.nnk, r.slot, r.nnk) ? c.m2 : c.m1);
  r.m2 = __uint_as_float(__reduce_min_sync(kFull, __float_as_uint(contrib)));
  return r;
}

// One float of a slot's geometry record (a strided view: float i of record
// s is p[4 s]), so that single fields read and write as from an array.
struct RecField {
  float* p;
  __device__ __forceinline__ float& operator[](int s) const { return p[4 * (int64_t)s]; }
};
struct RecInt {
  int* p;
  __device__ __forceinline__ int& operator[](int s) const { return p[4 * (int64_t)s]; }
};
struct RecByte {
  int8_t* p;
  __device__ __forceinline__ int8_t& operator[](int s) const { return p[16 * (int64_t)s]; }
};

// Per-event large workspace: pointers into the event's region of
// large_ws_bytes(N) bytes.  The window scans read a member's coordinates and
// neighbour interval together, so those four floats sit in one 16 B record
// per slot (one sector per lane for a warp's gather, not four); its
// neighbour, key interval, kind and liveness in a second one.
struct LargeWs {
  float4* geo;                           // [N] rap32, phi32, nlo, nhi
  RecField rap32, phi32, nlo, nhi;       // views of geo's fields
  int4* meta;                            // [N] nn, klo, khi (float bits), flags (byte 0 pair, byte 1 alive)
  RecInt nn;                             // views of meta's fields
  RecField klo, khi;
  RecByte pair, alive;
  float *wlo, *whi;                                           // [N]
  int *tile, *pos;                                            // [N]
  int* rc;                                                    // [N] slots whose neighbour this is
  int* members;                                               // [N + kListSlack * MT]
  int *t_start, *t_count;                                     // [MT] (the kernel points these
  TileSum* tsum;                                              // [MT]  three at shared memory)
  int max_tiles;                                              // MT
  int list_cap;                                               // bound of one tile's list length
};

__host__ __device__ __forceinline__ int large_max_tiles(int N) { return (N / 8 < kMaxTiles) ? N / 8 : kMaxTiles; }

__host__ __device__ __forceinline__ int64_t large_ws_bytes(int N) {
  const int64_t MT = large_max_tiles(N);
  const int64_t head = 52 * (int64_t)N;  // two 16 B records, two floats and three ints per slot
  return head + 4 * ((int64_t)N + kListSlack * MT) + 2 * 4 * MT + 16 + 32 * MT;
}

__device__ __forceinline__ LargeWs large_ws(unsigned char* base, int N) {
  LargeWs L;
  const int MT = large_max_tiles(N);
  float* f = reinterpret_cast<float*>(base);
  L.geo = reinterpret_cast<float4*>(f);  // 16 B aligned: the region starts at a multiple of 96 B
  L.rap32 = RecField{f};
  L.phi32 = RecField{f + 1};
  L.nlo = RecField{f + 2};
  L.nhi = RecField{f + 3};
  L.meta = reinterpret_cast<int4*>(f + 4 * N);
  int* mi = reinterpret_cast<int*>(L.meta);
  L.nn = RecInt{mi};
  L.klo = RecField{f + 4 * N + 1};
  L.khi = RecField{f + 4 * N + 2};
  L.pair = RecByte{reinterpret_cast<int8_t*>(mi + 3)};
  L.alive = RecByte{reinterpret_cast<int8_t*>(mi + 3) + 1};
  L.wlo = f + 8 * N;
  L.whi = f + 9 * N;
  int* i = reinterpret_cast<int*>(f + 10 * N);
  L.tile = i;
  L.pos = i + N;
  L.rc = i + 2 * N;
  int* m = i + 3 * N;
  L.members = m;
  L.t_start = m + N + kListSlack * MT;
  L.t_count = L.t_start + MT;
  const uintptr_t ts = (reinterpret_cast<uintptr_t>(L.t_count + MT) + 15) & ~uintptr_t(15);
  L.tsum = reinterpret_cast<TileSum*>(ts);
  L.max_tiles = MT;
  L.list_cap = N + kTileSlackMax;
  return L;
}

struct TiledShared {
  static constexpr int W = kTiledT / 32;
  double rmin, inv_side_r, inv_side_phi;
  int nrap, nphi, nt, slack;
  int rc_a_old, rc_drop;  // referrer-count updates of the step
  int ta_u, ta_v;  // tile of the new jet (rapidity and azimuth index)
  Cand wcand[W];
  Arg wexact[W];
  Cert wcert[W];
  Cert rcert[kTiledTargets][W];
  int rlist[kMaxListed];
  int n_rescan;
  int win_next;  // the window pass's next chunk of list positions (S3)
  int dirty[kMaxDirty];
  int n_dirty;
  unsigned dirty_bits[kMaxTiles / 32];
  int event, ctl_njets;
  double red[3][W];
  int scan_tmp[W];
  TilePart part;  // the new jet's tile without the new jet (S3c)
  // the event's tile lists' ranges and the tile summaries (LargeWs points here)
  int t_start[kSmemTiles], t_count[kSmemTiles];
  TileSum tsum[kSmemTiles];
};

__device__ __forceinline__ int tile_u(const TiledShared& S, double rap) {
  const int u = (int)floor((rap - S.rmin) * S.inv_side_r);
  return u < 0 ? 0 : (u >= S.nrap ? S.nrap - 1 : u);
}

__device__ __forceinline__ int tile_v(const TiledShared& S, double phi) {
  const int v = (int)floor(phi * S.inv_side_phi);
  return v < 0 ? 0 : (v >= S.nphi ? S.nphi - 1 : v);
}

// The distinct tiles of the 3x3 window around tile t.
__device__ __forceinline__ int window_tiles(const TiledShared& S, int t, int* out) {
  const int u = t / S.nphi, v = t - u * S.nphi;
  int k = 0;
  for (int du = -1; du <= 1; ++du) {
    const int uu = u + du;
    if (uu < 0 || uu >= S.nrap) continue;
    if (S.nphi <= 3) {
      for (int vv = 0; vv < S.nphi; ++vv) out[k++] = uu * S.nphi + vv;
    } else {
      for (int dv = -1; dv <= 1; ++dv) {
        int vv = v + dv;
        vv = vv < 0 ? vv + S.nphi : (vv >= S.nphi ? vv - S.nphi : vv);
        out[k++] = uu * S.nphi + vv;
      }
    }
  }
  return k;
}

// Union of the windows of tiles t1 and t2 (t2 < 0: t1's window only).
__device__ __forceinline__ int window_union(const TiledShared& S, int t1, int t2, int* out) {
  int nw = window_tiles(S, t1, out);
  if (t2 >= 0 && t2 != t1) {
    int more[kMaxWindowTiles];
    const int nm = window_tiles(S, t2, more);
    for (int k = 0; k < nm; ++k) {
      bool dup = false;
      for (int q = 0; q < kMaxWindowTiles; ++q) dup |= (q < nw && out[q] == more[k]);
      if (!dup) out[nw++] = more[k];
    }
  }
  return nw;
}

__device__ __forceinline__ bool tiles_adjacent(const TiledShared& S, int t1, int t2) {
  const int u1 = t1 / S.nphi, u2 = t2 / S.nphi;
  if (abs(u1 - u2) > 1) return false;
  if (S.nphi <= 3) return true;
  const int dv = abs((t1 - u1 * S.nphi) - (t2 - u2 * S.nphi));
  return dv <= 1 || dv == S.nphi - 1;
}

// Window scans.  The start and length of every tile of a window are read up
// front (independent loads), then the members are visited in passes: in a
// pass a thread takes the member at the same index of every tile, so that the
// loads for one member of each tile are in flight together.  A length is
// clamped to what a list can hold, so no scan is longer than the list area.
// Each thread reads the lengths itself: a list that grows meanwhile (an
// append in S3a) only adds or drops its last member, the new jet, which every
// caller skips by name.
template <int NT>
struct TileRanges {
  int start[NT], len[NT], tile[NT];
  int maxlen;
};

template <int NT>
__device__ __forceinline__ TileRanges<NT> tile_ranges(const LargeWs& L, const int* tiles, int nw) {
  TileRanges<NT> r;
  r.maxlen = 0;
#pragma unroll
  for (int k = 0; k < NT; ++k) {
    r.tile[k] = k < nw ? tiles[k] : 0;
    r.start[k] = k < nw ? L.t_start[r.tile[k]] : 0;
    const int m = k < nw ? L.t_count[r.tile[k]] : 0;
    r.len[k] = min(max(m, 0), L.list_cap);
    r.maxlen = max(r.maxlen, r.len[k]);
  }
  return r;
}

__device__ __forceinline__ double dr2_ws(const Ws& g, int s, int t) {
  return dr2_64(g.at(kRap, s), g.at(kPhi, s), g.at(kRap, t), g.at(kPhi, t));
}

// Key interval (or exact key) of slot t from its neighbour and distance interval.
__device__ __forceinline__ void set_key_large(const LargeWs& L, const EventCtx& X, int t) {
  const int nn = L.nn[t];
  if (nn < 0) {
    L.klo[t] = L.wlo[t];
    L.khi[t] = L.whi[t];
    L.pair[t] = 0;
    return;
  }
  float klo, khi;
  const int kind = key_interval(L.wlo[t], L.whi[t], L.wlo[nn], L.whi[nn], L.nlo[t], L.nhi[t], X.ilo, X.ihi, klo, khi);
  if (kind >= 0) {
    L.klo[t] = klo;
    L.khi[t] = khi;
    L.pair[t] = (int8_t)kind;
    return;
  }
  const double wt = X.g.at(kW, t);
  const double dp = pair_distance(wt, X.g.at(kW, nn), dr2_ws(X.g, t, nn), X.inv_r2);
  const bool is_pair = dp < wt;
  const double key = is_pair ? dp : wt;
  L.pair[t] = is_pair ? 1 : 0;
  L.klo[t] = fjk_to_f32(key, 1);
  L.khi[t] = fjk_to_f32(key, 2);
}

__device__ __forceinline__ double exact_key_large(const LargeWs& L, const EventCtx& X, int t) {
  if (!L.pair[t]) return L.klo[t] == L.khi[t] ? (double)L.klo[t] : X.g.at(kW, t);
  const int nn = L.nn[t];
  return pair_distance(X.g.at(kW, t), X.g.at(kW, nn), dr2_ws(X.g, t, nn), X.inv_r2);
}

// Bounds of dR2(t, u) from the FP32 filter's [lo, hi]; when that interval is
// wide (close pairs: the filter's error is absolute) the FP64 value is taken
// instead, so that the key intervals built on it stay narrow and the argmin
// certificates rarely fail.
__device__ __forceinline__ void tight_dr2(const EventCtx& X, int t, int u, float lo, float hi, float& lo_out,
                                          float& hi_out) {
  if (hi - lo <= lo * 0x1p-16f) {
    lo_out = lo;
    hi_out = hi;
  } else {
    const double d = dr2_ws(X.g, t, u);
    lo_out = fjk_to_f32(d, 1);
    hi_out = fjk_to_f32(d, 2);
  }
}

// Certificate partial of slot t's nearest neighbour over the window of its
// tile, visited by `nthreads` threads starting at `first`; slots t, skip1 and
// skip2 and tombstones are skipped.
__device__ __forceinline__ void window_cert(const TiledShared& S, const LargeWs& L, const EventCtx& X, int t,
                                            int first, int nthreads, int skip1, int skip2, Cert& c) {
  int tiles[kMaxWindowTiles];
  const int nw = window_tiles(S, L.tile[t], tiles);
  const float rt = L.rap32[t], pt = L.phi32[t];
  const TileRanges<kMaxWindowTiles> R = tile_ranges<kMaxWindowTiles>(L, tiles, nw);
  for (int i = first; i < R.maxlen; i += nthreads) {
    int u[kMaxWindowTiles];
    float r[kMaxWindowTiles], ph[kMaxWindowTiles];
#pragma unroll
    for (int k = 0; k < kMaxWindowTiles; ++k) u[k] = i < R.len[k] ? L.members[R.start[k] + i] : -1;
#pragma unroll
    for (int k = 0; k < kMaxWindowTiles; ++k) {
      if (u[k] >= 0) {
        const float2 g2 = *reinterpret_cast<const float2*>(L.geo + u[k]);
        r[k] = g2.x;
        ph[k] = g2.y;
      }
    }
#pragma unroll
    for (int k = 0; k < kMaxWindowTiles; ++k) {
      if (u[k] < 0 || u[k] == t || u[k] == skip1 || u[k] == skip2) continue;
      float lo, hi;
      dr2_32(rt, pt, r[k], ph[k], X.bd, lo, hi);
      cert_add(c, lo, hi, u[k]);
    }
  }
}

// Slot t's neighbour from a combined certificate over the same candidates
// (window minus skip1/skip2, plus `extra` when >= 0).  Near-ties are settled
// in FP64 with the lowest slot first.  Whole warp.
__device__ __forceinline__ int resolve_large(const TiledShared& S, const LargeWs& L, const EventCtx& X, int t,
                                             const Cert& c, int skip1, int skip2, int extra, float& lo_out,
                                             float& hi_out) {
  if (c.i1 < 0) {
    lo_out = hi_out = __int_as_float(0x7f800000);
    return -1;
  }
  if (cert_ok(c)) {
    tight_dr2(X, t, c.i1, c.m1, c.u1, lo_out, hi_out);
    return c.i1;
  }
  const int lane = threadIdx.x & 31;
  unsigned long long bk = ~0ull;
  int bi = 0x7fffffff;
  const float rt = L.rap32[t], pt = L.phi32[t];
  auto consider = [&](int u) {
    float lo, hi;
    dr2_32(rt, pt, L.rap32[u], L.phi32[u], X.bd, lo, hi);
    if (lo <= c.u1) {
      const unsigned long long k = dbits(dr2_ws(X.g, t, u));
      if (arg_less(k, u, bk, bi)) {
        bk = k;
        bi = u;
      }
    }
  };
  int tiles[kMaxWindowTiles];
  const int nw = window_tiles(S, L.tile[t], tiles);
  for (int k = 0; k < nw; ++k) {
    const int tt = tiles[k];
    const int base = L.t_start[tt], m = L.t_count[tt];
    for (int i = lane; i < m; i += 32) {
      const int u = L.members[base + i];
      if (u >= 0 && u != t && u != skip1 && u != skip2 && u != extra) consider(u);
    }
  }
  if (extra >= 0 && lane == 0) consider(extra);
  const Arg r = arg_warp(bk, bi, bi);
  const double d = __longlong_as_double((long long)r.key);
  lo_out = fjk_to_f32(d, 1);
  hi_out = fjk_to_f32(d, 2);
  return r.idx;
}

// Summary parts of the members of tile tt other than `skip` (whole warp;
// every lane receives them): the smallest key lower bound m1 and its slot x
// (the lowest among equal bounds) with x's key upper bound and neighbour
// field, and mo, the smallest lower bound of the other members without x's
// mutual partner.  Each lane keeps its two smallest bounds with their slots
// and the third smallest bound, reading four members per pass; x's neighbour
// field (and its neighbour's, to recognise a mutual partner) is read once at
// the end.  When x's neighbour is `skip` (a slot whose state another warp may
// be writing) its fields are not read: mo then leaves out x alone, and
// merge_skipped decides the partner once skip's state is known.
__device__ __forceinline__ TilePart tile_part(const LargeWs& L, int tt, int skip) {
  constexpr int B = 4;
  const int lane = threadIdx.x & 31;
  const float inf = __int_as_float(0x7f800000);
  float m1 = inf, m2 = inf, m3 = inf;
  int s1 = -1, s2 = -1;
  const int base = L.t_start[tt], m = min(max(L.t_count[tt], 0), L.list_cap);
  for (int i0 = lane; i0 < m; i0 += 32 * B) {
    int u[B];
    float lo[B];
#pragma unroll
    for (int q = 0; q < B; ++q) {
      u[q] = i0 + 32 * q < m ? L.members[base + i0 + 32 * q] : -1;
      if (u[q] == skip) u[q] = -1;
    }
#pragma unroll
    for (int q = 0; q < B; ++q) lo[q] = u[q] >= 0 ? L.klo[u[q]] : inf;
#pragma unroll
    for (int q = 0; q < B; ++q) {
      if (u[q] < 0) continue;
      if (lo[q] < m1 || (lo[q] == m1 && (unsigned)u[q] < (unsigned)s1)) {
        m3 = m2;
        m2 = m1;
        s2 = s1;
        m1 = lo[q];
        s1 = u[q];
      } else if (lo[q] < m2 || (lo[q] == m2 && (unsigned)u[q] < (unsigned)s2)) {
        m3 = m2;
        m2 = lo[q];
        s2 = u[q];
      } else {
        m3 = fminf(m3, lo[q]);
      }
    }
  }
  const unsigned mb = __reduce_min_sync(kFull, __float_as_uint(m1));
  const bool at_min = __float_as_uint(m1) == mb && s1 >= 0;
  const unsigned sb = __reduce_min_sync(kFull, at_min ? (unsigned)s1 : 0xffffffffu);
  const int x = sb == 0xffffffffu ? -1 : (int)sb;
  int nnk = kNoNeighbour, p = -1;
  float u1 = inf;
  if (lane == 0 && x >= 0) {
    const int4 mx = L.meta[x];
    const int nx = mx.x;
    const bool px = (int8_t)mx.w != 0;
    u1 = __int_as_float(mx.z);
    nnk = (nx < 0 ? kNoNeighbour : nx) | (px ? (int)kPairBit : 0);
    if (px && nx >= 0 && nx != skip) {
      const int4 mn = L.meta[nx];
      if ((int8_t)mn.w != 0 && mn.x == x) p = nx;
    }
  }
  p = __shfl_sync(kFull, p, 0);
  // smallest bound of the lane's members other than the winner and its partner
  const float contrib = (s1 >= 0 && s1 != x && s1 != p) ? m1 : (s2 >= 0 && s2 != x && s2 != p) ? m2 : m3;
  const float mo = __uint_as_float(__reduce_min_sync(kFull, __float_as_uint(contrib)));
  return TilePart{__uint_as_float(mb), x, __shfl_sync(kFull, u1, 0), __shfl_sync(kFull, nnk, 0), mo};
}

// Summary of tile tt (whole warp).
__device__ __forceinline__ void tile_summary(const LargeWs& L, int tt) {
  const TilePart P = tile_part(L, tt, -1);
  if ((threadIdx.x & 31) == 0) L.tsum[tt] = TileSum{P.m1, P.x, P.u1, P.mo, P.nnk, 0, 0, 0};
}

// The summary of a tile from the parts of its members other than slot a
// (tile_part with skip = a) and a's own key and neighbour field.  a wins by
// (klo, slot); the second bound leaves out the winner's mutual partner, and
// two slots are mutual partners exactly when each one's neighbour field names
// the other with the pair bit -- so no further state is read.
//   a wins: the smallest other bound is P's winner's, unless that winner is
//     a's mutual partner; then its field names a, P.mo left out P.x alone,
//     and P.mo is the bound.
//   P.x wins: P.mo left out P.x and its partner, a included when P.x's field
//     does not name a (then a is neither); when it names a, P.mo left out P.x
//     alone, and a's bound counts unless a is the mutual partner.
__host__ __device__ __forceinline__ TileSum merge_skipped(const TilePart& P, int a, float ka, float ua, int nnka) {
  const int a_pair = (int)((unsigned)a | kPairBit);
  if (P.x < 0 || ka < P.m1 || (ka == P.m1 && (unsigned)a < (unsigned)P.x)) {
    const bool mutual = P.x >= 0 && P.nnk == a_pair && nnka == (int)((unsigned)P.x | kPairBit);
    return TileSum{ka, a, ua, mutual ? P.mo : P.m1, nnka, 0, 0, 0};
  }
  const bool mutual = P.nnk == a_pair && nnka == (int)((unsigned)P.x | kPairBit);
  return TileSum{P.m1, P.x, P.u1, mutual ? P.mo : fminf(P.mo, ka), P.nnk, 0, 0, 0};
}

// Block-wide rebuild of the tile lists from the live slots (S.slack free
// entries per tile, filled with tombstones) and of every tile summary.
__device__ inline void rebuild_tiles(TiledShared& S, const LargeWs& L, int N, bool summaries = true) {
  constexpr int W = kTiledT / 32;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int t = tid; t < S.nt; t += kTiledT) L.t_count[t] = 0;
  __syncthreads();
  for (int s = tid; s < N; s += kTiledT)
    if (L.alive[s]) atomicAdd(&L.t_count[L.tile[s]], 1);
  __syncthreads();
  // exclusive scan of (count + slack) over the tiles, kTiledT at a time
  int carry = 0;
  for (int base = 0; base < S.nt; base += kTiledT) {
    const int t = base + tid;
    const int v = (t < S.nt) ? L.t_count[t] + S.slack : 0;
    int incl = v;
    for (int o = 1; o < 32; o <<= 1) {
      const int x = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += x;
    }
    if (lane == 31) S.scan_tmp[warp] = incl;
    __syncthreads();
    int wpre = 0, total = 0;
    for (int k = 0; k < W; ++k) {
      if (k < warp) wpre += S.scan_tmp[k];
      total += S.scan_tmp[k];
    }
    if (t < S.nt) {
      L.t_start[t] = carry + wpre + incl - v;
      L.t_count[t] = 0;
    }
    carry += total;
    __syncthreads();
  }
  for (int s = tid; s < N; s += kTiledT) {
    if (!L.alive[s]) continue;
    const int t = L.tile[s];
    const int p = atomicAdd(&L.t_count[t], 1);
    L.members[L.t_start[t] + p] = s;
    L.pos[s] = p;
  }
  __syncthreads();
  for (int t = warp; t < S.nt; t += W) {
    const int end = L.t_start[t] + L.t_count[t];
    for (int i = lane; i < S.slack; i += 32) L.members[end + i] = -1;
  }
  __syncthreads();
  if (summaries) {
    for (int t = warp; t < S.nt; t += W) tile_summary(L, t);
    __syncthreads();
  }
}

__device__ __forceinline__ void mark_dirty(TiledShared& S, int t) {
  const unsigned bit = 1u << (t & 31);
  const unsigned old = atomicOr(&S.dirty_bits[t >> 5], bit);
  if (!(old & bit)) {
    const int k = atomicAdd(&S.n_dirty, 1);
    if (k < kMaxDirty) S.dirty[k] = t;
  }
}

// A whole warp rescans slot t's window (lists up to date) and stores its
// neighbour and key.
__device__ __forceinline__ void rescan_warp(TiledShared& S, const LargeWs& L, const EventCtx& X, int t, int skip) {
  const int lane = threadIdx.x & 31;
  Cert x = cert_empty();
  window_cert(S, L, X, t, lane, 32, skip, -1, x);
  x = cert_warp(x);
  float lo, hi;
  const int nn = resolve_large(S, L, X, t, x, skip, -1, -1, lo, hi);
  if (lane == 0) {
    if (nn >= 0) atomicAdd(&L.rc[nn], 1);  // t's old neighbour was a merged slot
    L.nn[t] = nn;
    L.nlo[t] = lo;
    L.nhi[t] = hi;
    set_key_large(L, X, t);
    mark_dirty(S, L.tile[t]);
  }
  __syncwarp();
}

__device__ inline void cluster_event_tiled(TiledShared& S, const BatchArgs& A, unsigned char* large_base, int e) {
  constexpr int T = kTiledT;
  constexpr int W = T / 32;
  constexpr int MW = 3;
  constexpr int TR = T - 32 * MW;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  int64_t off;
  EventCtx X;
  event_range(A, e, off, X.N);
  X.algo = A.algo ? A.algo[e] : A.algo_all;
  const double R = A.radius ? A.radius[e] : A.r_all;
  X.inv_r2 = 1.0 / (R * R);
  X.ilo = fjk_to_f32(X.inv_r2, 1);
  X.ihi = fjk_to_f32(X.inv_r2, 2);
  X.g.base = A.ws + off;
  X.g.stride = A.ws_stride;
  const Ws& g = X.g;
  const int N = X.N;
  // event e's region starts kLargeWsBytesPerParticle * offsets[e] bytes in
  LargeWs L = large_ws(large_base + off * kLargeWsBytesPerParticle, N);
  L.t_start = S.t_start;
  L.t_count = S.t_count;
  L.tsum = S.tsum;

  // ---- load and kinematics; rapidity range
  double rlo = 1e300, rhi = -1e300, amax = 0.0;
  for (int s = tid; s < N; s += T) {
    const double* p = A.p4 + (off + s) * A.p4_stride;
    const double px = p[0], py = p[1], pz = p[2], E = p[3];
    const Kin kin = kinematics(px, py, pz, E, X.algo);
    g.at(kPx, s) = px;
    g.at(kPy, s) = py;
    g.at(kPz, s) = pz;
    g.at(kE, s) = E;
    g.at(kRap, s) = kin.rap;
    g.at(kPhi, s) = kin.phi;
    g.at(kW, s) = kin.w;
    L.rap32[s] = fjk_to_f32(kin.rap, 0);
    L.phi32[s] = fjk_to_f32(kin.phi, 0);
    L.wlo[s] = fjk_to_f32(kin.w, 1);
    L.whi[s] = fjk_to_f32(kin.w, 2);
    L.alive[s] = 1;
    rlo = fmin(rlo, kin.rap);
    rhi = fmax(rhi, kin.rap);
    amax = fmax(amax, fabs(kin.rap));
    if (A.owner) A.owner[off + s] = s;  // union-find parent by label
  }
  for (int o = 16; o; o >>= 1) {
    rlo = fmin(rlo, __shfl_xor_sync(kFull, rlo, o));
    rhi = fmax(rhi, __shfl_xor_sync(kFull, rhi, o));
    amax = fmax(amax, __shfl_xor_sync(kFull, amax, o));
  }
  if (lane == 0) {
    S.red[0][warp] = rlo;
    S.red[1][warp] = rhi;
    S.red[2][warp] = amax;
  }
  for (int k = tid; k < kMaxTiles / 32; k += T) S.dirty_bits[k] = 0;
  __syncthreads();
  if (tid == 0) {
    double lo = 1e300, hi = -1e300;
    for (int k = 0; k < W; ++k) {
      lo = fmin(lo, S.red[0][k]);
      hi = fmax(hi, S.red[1][k]);
    }
    lo = fmax(lo, -15.0);
    hi = fmin(hi, 15.0);
    if (!(hi >= lo)) hi = lo;
    // tile side: at least R (times the tuning factor), and large enough that
    // a tile holds about kTileMembers particles on average, so that sparse
    // events do not scan mostly empty windows
    const double side_r = R * fmax(A.tile_factor, 1.0) * (1.0 + 1e-4) + 1e-5;
    const double area = fmax(hi - lo, side_r) * 6.283185307179586;
    const double side_min = fmax(side_r, sqrt(area * kTileMembers / (double)N));
    int nphi = (int)fmin(floor(6.283185307179586 / side_min), 4096.0);
    nphi = nphi < 1 ? 1 : nphi;
    int nrap = (int)fmin(floor((hi - lo) / side_min), 4096.0);
    nrap = nrap < 1 ? 1 : nrap;
    // coarser tiles are still correct, only slower
    while (nrap * nphi > min(L.max_tiles, kSmemTiles)) {
      if (nrap > 1)
        nrap = (nrap + 1) / 2;
      else
        nphi = (nphi + 1) / 2;
    }
    S.nrap = nrap;
    S.nphi = nphi;
    S.nt = nrap * nphi;
    S.slack = min(kTileSlackMax, kListSlack * L.max_tiles / S.nt);
    S.rmin = lo;
    S.inv_side_r = (double)nrap / fmax(hi - lo, side_min);
    S.inv_side_phi = (double)nphi / 6.283185307179586;
    S.ctl_njets = 0;
    S.n_rescan = 0;
    S.n_dirty = 0;
    S.win_next = 0;
  }
  {
    double rmax = 0.0;
    for (int k = 0; k < W; ++k) rmax = fmax(rmax, S.red[2][k]);
    X.bd = make_bound(rmax);
  }
  __syncthreads();
  for (int s = tid; s < N; s += T) L.tile[s] = tile_u(S, g.at(kRap, s)) * S.nphi + tile_v(S, g.at(kPhi, s));
  __syncthreads();
  // lists only: the summaries read neighbours and keys, which do not exist yet
  rebuild_tiles(S, L, N, false);

  // ---- initial nearest neighbours within the windows
  for (int s = tid; s < N; s += T) L.rc[s] = 0;
  __syncthreads();
  for (int t = tid; t < N; t += T) {
    Cert c = cert_empty();
    window_cert(S, L, X, t, 0, 1, -1, -1, c);
    int nn = c.i1;
    float nlo = c.m1, nhi = c.u1;
    if (nn >= 0 && cert_ok(c)) tight_dr2(X, t, nn, c.m1, c.u1, nlo, nhi);
    if (nn >= 0 && !cert_ok(c)) {
      unsigned long long bk = ~0ull;
      int bi = 0x7fffffff;
      int tiles[kMaxWindowTiles];
      const int nw = window_tiles(S, L.tile[t], tiles);
      const float rt = L.rap32[t], pt = L.phi32[t];
      for (int k = 0; k < nw; ++k) {
        const int base = L.t_start[tiles[k]], m = L.t_count[tiles[k]];
        for (int i = 0; i < m; ++i) {
          const int u = L.members[base + i];
          if (u < 0 || u == t) continue;
          float lo, hi;
          dr2_32(rt, pt, L.rap32[u], L.phi32[u], X.bd, lo, hi);
          if (lo <= c.u1) {
            const unsigned long long du = dbits(dr2_ws(g, t, u));
            if (arg_less(du, u, bk, bi)) {
              bk = du;
              bi = u;
            }
          }
        }
      }
      nn = bi;
      const double d = __longlong_as_double((long long)bk);
      nlo = fjk_to_f32(d, 1);
      nhi = fjk_to_f32(d, 2);
    }
    L.nn[t] = nn;
    L.nlo[t] = nlo;
    L.nhi[t] = nhi;
    if (nn >= 0) atomicAdd(&L.rc[nn], 1);
  }
  __syncthreads();
  for (int t = tid; t < N; t += T) set_key_large(L, X, t);
  __syncthreads();
  for (int t = warp; t < S.nt; t += W) tile_summary(L, t);
  __syncthreads();

  // ---- clustering steps
  int n = N;
  int step = 0;
  FJG_PH(long long ph_rb = 0, ph_s1 = 0, ph_s2 = 0, ph_s3a = 0, ph_s3b = 0, ph_s3c = 0, ph_kin = 0, ph_det = 0;
         long long ph_tg = 0, ph_tgs = 0, ph_lu = 0, ph_tt = 0, ph_wp = 0, ph_ra = 0, ph_sa = 0, ph_so = 0;)
  while (n > 0) {
    FJG_PH(const long long ph0 = clock64();)
    if (step > 0 && step % S.slack == 0) rebuild_tiles(S, L, N);
    FJG_PH(const long long phr = clock64(); ph_rb += phr - ph0;)

    // S1: argmin over the tile summaries (slot order breaks ties)
    Cand mine = cand_empty();
    for (int t = tid; t < S.nt; t += T) {
      const TileSum ts = L.tsum[t];
      cand_merge(mine, Cand{ts.m1, ts.slot, ts.u1, ts.nnk, ts.m2});
    }
    {
      const Cand wc = cand_warp(mine);
      if (lane == 0) S.wcand[warp] = wc;
    }
    __syncthreads();  // B1
    int c;
    {
      const Cand x = cand_warp((lane < W) ? S.wcand[lane] : cand_empty());
      c = x.slot;
      const float u1 = x.u1, m2 = x.m2;
      if (c >= 0 && !(u1 < m2)) {
        // near-tie: exact keys of every slot whose lower bound is <= u1
        unsigned long long bk = ~0ull;
        int bi = 0x7fffffff;
        for (int tt = warp; tt < S.nt; tt += W) {
          if (!(L.tsum[tt].m1 <= u1)) continue;
          const int base = L.t_start[tt], m = L.t_count[tt];
          for (int i = lane; i < m; i += 32) {
            const int t = L.members[base + i];
            if (t >= 0 && L.klo[t] <= u1) {
              const unsigned long long kk = dbits(exact_key_large(L, X, t));
              if (arg_less(kk, t, bk, bi)) {
                bk = kk;
                bi = t;
              }
            }
          }
        }
        const Arg wa = arg_warp(bk, bi, bi);
        if (lane == 0) S.wexact[warp] = wa;
        __syncthreads();
        const Arg y = (lane < W) ? S.wexact[lane] : Arg{~0ull, 0x7fffffff, -1};
        c = arg_warp(y.key, y.label, y.idx).idx;
        __syncthreads();
      }
    }
    if (c < 0) {
      if (tid == 0) raise_event_status(A, e, kStatusInternal);
      break;
    }

    // S2
    FJG_PH(const long long ph1 = clock64(); ph_s1 += ph1 - phr;)
    const bool pair = L.pair[c] != 0 && L.nn[c] >= 0;
    const int j = pair ? L.nn[c] : -1;
    const int a = pair ? min(c, j) : -1;
    const int b = pair ? max(c, j) : c;
    const int tile_c = L.tile[c], tile_j = pair ? L.tile[j] : -1;

    if (warp < MW) {
      double pxc = 0, pyc = 0, pzc = 0, Ec = 0, pxj = 0, pyj = 0, pzj = 0, Ej = 0;
      double rc = 0, fc = 0, wc = 0, rj = 0, fj = 0, wj = 0;
      if (lane == 0) {
        pxc = g.at(kPx, c);
        pyc = g.at(kPy, c);
        pzc = g.at(kPz, c);
        Ec = g.at(kE, c);
        wc = g.at(kW, c);
        if (pair) {
          pxj = g.at(kPx, j);
          pyj = g.at(kPy, j);
          pzj = g.at(kPz, j);
          Ej = g.at(kE, j);
          wj = g.at(kW, j);
          rc = g.at(kRap, c);
          fc = g.at(kPhi, c);
          rj = g.at(kRap, j);
          fj = g.at(kPhi, j);
        }
      }
      __syncwarp();
      named_sync(2, 32 * MW);  // every merge warp has read c and j
      FJG_PH(const long long pk0 = clock64();)
      if (pair) {
        const double px = __dadd_rn(pxc, pxj), py = __dadd_rn(pyc, pyj);
        if (lane == 0 && warp == 0) {
          const double phi = fjk_phi(px, py);
          g.at(kPhi, a) = phi;
          L.phi32[a] = fjk_to_f32(phi, 0);
          S.ta_v = tile_v(S, phi);
        }
        if (lane == 0 && warp == 1) {
          const double pz = __dadd_rn(pzc, pzj), E = __dadd_rn(Ec, Ej);
          const double rap = fjk_rap(px, py, pz, E);
          g.at(kPx, a) = px;
          g.at(kPy, a) = py;
          g.at(kPz, a) = pz;
          g.at(kE, a) = E;
          g.at(kRap, a) = rap;
          L.rap32[a] = fjk_to_f32(rap, 0);
          S.ta_u = tile_u(S, rap);
        }
        if (lane == 0 && warp == 2) {
          const double w = fjk_weight(px, py, X.algo);
          g.at(kW, a) = w;
          L.wlo[a] = fjk_to_f32(w, 1);
          L.whi[a] = fjk_to_f32(w, 2);
          const double d = pair_distance(wc, wj, dr2_64(rc, fc, rj, fj), X.inv_r2);
          if (A.history) A.history[off + step] = StepRec{a, b, d};
          if (A.owner) A.owner[off + b] = a;
        }
      } else if (lane == 0 && warp == 2) {
        const int nj = S.ctl_njets;
        double* jo = A.jets + (off + nj) * 4;
        jo[0] = pxc;
        jo[1] = pyc;
        jo[2] = pzc;
        jo[3] = Ec;
        A.jet_label[off + nj] = c;
        if (A.history) A.history[off + step] = StepRec{c, -1, wc};
        if (A.owner) A.owner[off + c] = -(nj + 1);
        S.ctl_njets = nj + 1;
      }
      FJG_PH(if (lane == 0) ph_kin += clock64() - pk0;)  // warp 1's (the rapidity chain) is reported
      __syncwarp();
    } else {
      // targets: live slots other than c, j whose neighbour is c or j; they
      // lie in the windows of c's and j's tiles.  The referrer counts say how
      // many there are (c's neighbour is j for a pair, and j's may be c):
      // without any, the scan is skipped (the same values for every thread)
      const int r0 = tid - 32 * MW;
      const int rcc = L.rc[c], rcj = pair ? L.rc[j] : 0, nnj = pair ? L.nn[j] : -1;
      const int expected = pair ? rcc + rcj - 1 - (nnj == c ? 1 : 0) : rcc;
      if (r0 == 0) {
        // referrer counts this step retires (applied after B2, read before
        // any update): the new jet's slot loses its old referrers (the
        // targets, which count again under their new neighbours), and the
        // merged slots' own old neighbours lose one each
        S.rc_a_old = pair ? (a == c ? rcc : rcj) : 0;
        S.rc_drop = pair ? ((nnj != c && nnj != j) ? nnj : -1) : L.nn[c];
      }
      if (expected > 0) {
        int tiles[2 * kMaxWindowTiles];
        const int nw = window_union(S, tile_c, tile_j, tiles);
        constexpr int NU = 2 * kMaxWindowTiles;
        const TileRanges<NU> R = tile_ranges<NU>(L, tiles, nw);
        for (int i = r0; i < R.maxlen; i += TR) {
          // the referrer counts say how many targets there are: once all are
          // found, the remaining passes would find none
          if (*(volatile int*)&S.n_rescan >= expected) break;
          int u[NU], nu[NU];
  #pragma unroll
          for (int k = 0; k < NU; ++k) u[k] = i < R.len[k] ? L.members[R.start[k] + i] : -1;
  #pragma unroll
          for (int k = 0; k < NU; ++k) nu[k] = u[k] >= 0 ? L.nn[u[k]] : -1;
  #pragma unroll
          for (int k = 0; k < NU; ++k) {
            if (u[k] < 0 || u[k] == c || u[k] == j) continue;
            if (nu[k] == c || (pair && nu[k] == j)) {
              const int p = atomicAdd(&S.n_rescan, 1);
              if (p < kMaxListed) S.rlist[p] = u[k];
              L.alive[u[k]] = 2;  // a target of this step (cleared after B3)
            }
          }
        }
        named_sync(1, TR);
        const int nr = min(S.n_rescan, kTiledTargets);
        for (int r = 0; r < nr; ++r) {
          Cert rc = cert_empty();
          window_cert(S, L, X, S.rlist[r], r0, TR, c, j, rc);
          const Cert wc = cert_warp(rc);
          if (lane == 0) S.rcert[r][warp] = wc;
        }
      }
      FJG_PH(if (r0 == 0) ph_det += clock64() - ph1;)
    }
    __syncthreads();  // B2
    FJG_PH(const long long ph2 = clock64(); ph_s2 += ph2 - ph1;)
    --n;
    ++step;
    if (n == 0) break;
    const int n_found = S.n_rescan;
    FJG_PH(ph_tg += n_found; ph_tgs += n_found > 0;)
    const int nr_all = min(n_found, kMaxListed);
    const int nr = min(nr_all, kTiledTargets);
    const int ta = pair ? S.ta_u * S.nphi + S.ta_v : -1;

    // S3a: tile lists (thread 0: a tombstone for b, and for a when it
    // changes tile, then an append); targets (one warp each)
    if (tid == 0) {
      FJG_PH(const long long q0 = clock64();)
      // every word the update reads is loaded before its first store: the
      // arrays are distinct, but the compiler cannot know that the stores to
      // the member lists leave them alone, and would otherwise wait for each
      // store before the next load (two L2 round trips instead of four)
      const int tb = L.tile[b], pb = L.pos[b];
      const int told = pair ? L.tile[a] : -1, pa = pair ? L.pos[a] : 0;
      const int cta = pair ? L.t_count[ta] : 0, sta = pair ? L.t_start[ta] : 0;
      const int sb = L.t_start[tb];
      const int sold = pair ? L.t_start[told] : 0;
      if (pair) atomicSub(&L.rc[a], S.rc_a_old);
      if (S.rc_drop >= 0) atomicSub(&L.rc[S.rc_drop], 1);
      L.members[sb + pb] = -1;
      L.alive[b] = 0;
      mark_dirty(S, tb);
      if (pair) {
        mark_dirty(S, told);
        if (ta != told) {
          L.members[sold + pa] = -1;
          L.members[sta + cta] = a;
          L.pos[a] = cta;
          L.tile[a] = ta;
          L.t_count[ta] = cta + 1;
          mark_dirty(S, ta);
        }
      }
      FJG_PH(ph_lu += clock64() - q0;)
    }
    // targets go to warps 1, 2, ... first: warp 0's thread 0 is busy above
    FJG_PH(const long long q1 = clock64();)
    for (int r = (warp + W - 1) % W; r < nr_all; r += W) {
      const int t = S.rlist[r];
      Cert x = cert_empty();
      if (r < nr)
        x = (lane >= MW && lane < W) ? S.rcert[r][lane] : cert_empty();
      else
        window_cert(S, L, X, t, lane, 32, c, j, x);
      const int extra = (pair && tiles_adjacent(S, L.tile[t], ta)) ? a : -1;
      if (extra >= 0 && lane == 0) {
        float lo, hi;
        dr2_32(L.rap32[t], L.phi32[t], L.rap32[a], L.phi32[a], X.bd, lo, hi);
        cert_add(x, lo, hi, a);
      }
      x = cert_warp(x);
      float lo, hi;
      const int nn = resolve_large(S, L, X, t, x, c, j, extra, lo, hi);
      if (lane == 0) {
        if (nn >= 0) atomicAdd(&L.rc[nn], 1);
        L.nn[t] = nn;
        L.nlo[t] = lo;
        L.nhi[t] = hi;
        set_key_large(L, X, t);
        mark_dirty(S, L.tile[t]);
      }
      __syncwarp();
    }
    FJG_PH(const long long q2 = clock64(); if (warp == 1 && lane == 0) ph_tt += q2 - q1;)
    // S3b, in the same phase: every slot of the new jet's window against the
    // new jet, beside the list update and the targets' searches (no barrier
    // between them).  This step's targets (alive == 2, set before B2) are
    // compared for the new jet's own search but not updated: their searches
    // offer them the new jet (`extra`).  Every other slot's neighbour,
    // intervals and key are written only here, the lists are read as the
    // targets' scans read them (see "Tile lists"), and the new jet's fields
    // were written before B2.
    if (pair) {
      Cert ca = cert_empty();
      int tiles[kMaxWindowTiles];
      const int nw = window_tiles(S, ta, tiles);
      const float ra = L.rap32[a], pa = L.phi32[a];
      constexpr int NT = kMaxWindowTiles;
      const TileRanges<NT> R = tile_ranges<NT>(L, tiles, nw);
      // list positions go out 32 at a time from a shared counter, so that
      // the warps that ran the list update or a target come late and take
      // fewer (each warp takes chunks until the longest list is covered)
      for (;;) {
        int base = 0;
        if (lane == 0) base = atomicAdd(&S.win_next, 32);
        base = __shfl_sync(kFull, base, 0);
        if (base >= R.maxlen) break;
        const int i = base + lane;
        int u[NT], cn[NT], al[NT];
        float r[NT], ph[NT], nl[NT], nh[NT];
#pragma unroll
        for (int k = 0; k < NT; ++k) u[k] = i < R.len[k] ? L.members[R.start[k] + i] : -1;
#pragma unroll
        for (int k = 0; k < NT; ++k) {
          if (u[k] >= 0) {
            const float4 g4 = L.geo[u[k]];
            r[k] = g4.x;
            ph[k] = g4.y;
            nl[k] = g4.z;
            nh[k] = g4.w;
            const int4 m4 = L.meta[u[k]];
            cn[k] = m4.x;
            al[k] = (int8_t)(m4.w >> 8);
          }
        }
#pragma unroll
        for (int k = 0; k < NT; ++k) {
          const int t = u[k];
          if (t < 0 || t == a || t == b) continue;
          float lo, hi;
          dr2_32(r[k], ph[k], ra, pa, X.bd, lo, hi);
          cert_add(ca, lo, hi, t);
          if (cn[k] == a || al[k] == 2) continue;
          bool closer;
          float ulo = lo, uhi = hi;
          if (cn[k] < 0 || hi < nl[k]) {
            closer = true;
            tight_dr2(X, t, a, lo, hi, ulo, uhi);
          } else if (lo > nh[k]) {
            closer = false;
          } else {
            const double da = dr2_ws(g, t, a);
            const double dc = dr2_ws(g, t, cn[k]);
            closer = da < dc || (da == dc && a < cn[k]);
            ulo = fjk_to_f32(da, 1);
            uhi = fjk_to_f32(da, 2);
          }
          if (closer) {
            if (cn[k] >= 0) atomicSub(&L.rc[cn[k]], 1);
            atomicAdd(&L.rc[a], 1);
            L.nn[t] = a;
            L.nlo[t] = ulo;
            L.nhi[t] = uhi;
            set_key_large(L, X, t);
            mark_dirty(S, R.tile[k]);
          }
        }
      }
      const Cert wc = cert_warp(ca);
      if (lane == 0) S.wcert[warp] = wc;
    }
    FJG_PH(if (tid == 0) ph_wp += clock64() - q2;)
    __syncthreads();  // B3: lists updated, listed targets done, the new jet's window compared
    FJG_PH(const long long ph3 = clock64(); ph_s3a += ph3 - ph2;)
    if (n_found > kMaxListed) {
      // more targets than listed (degenerate inputs, e.g. repeated
      // particles): the unlisted ones (still flagged) are searched again
      // with the lists up to date, which offers them the new jet
      int tiles[2 * kMaxWindowTiles];
      const int nw = window_union(S, tile_c, tile_j, tiles);
      for (int k = warp; k < nw; k += W) {
        const int base = L.t_start[tiles[k]], m = L.t_count[tiles[k]];
        for (int i0 = 0; i0 < m; i0 += 32) {
          const int i = i0 + lane;
          const int u = (i < m) ? L.members[base + i] : -1;
          const bool hit = u >= 0 && u != a && u != b && L.alive[u] == 2;
          unsigned ball = __ballot_sync(kFull, hit);
          while (ball) {
            const int src = __ffs(ball) - 1;
            ball &= ball - 1;
            const int t = __shfl_sync(kFull, u, src);
            bool listed = false;
            for (int q = lane; q < kMaxListed; q += 32) listed |= S.rlist[q] == t;
            if (!__any_sync(kFull, listed)) {
              rescan_warp(S, L, X, t, b);
              if (lane == 0) L.alive[t] = 1;
            }
          }
        }
      }
      __syncthreads();
    }
    for (int r = tid; r < nr_all; r += T) L.alive[S.rlist[r]] = 1;  // the listed targets' flags
    FJG_PH(const long long ph4 = clock64(); ph_s3b += ph4 - ph3;)
    // S3c: the new jet's neighbour (warp 0, then its tile's summary) and the
    // other changed tiles' summaries (the remaining warps)
    const int nd = S.n_dirty;
    FJG_PH(const long long q5 = clock64();)
    if (pair && warp == 1) {
      // the new jet's tile without the new jet, while warp 0 resolves it
      // (tile_part reads none of the new jet's state)
      const TilePart P = tile_part(L, ta, a);
      if (lane == 0) S.part = P;
      named_sync(3, 64);
    }
    if (pair && warp == 0) {
      FJG_PH(const long long q3 = clock64();)
      Cert x = (lane < W) ? S.wcert[lane] : cert_empty();
      x = cert_warp(x);
      float lo, hi;
      const int nn = resolve_large(S, L, X, a, x, b, -1, -1, lo, hi);
      int nnka = kNoNeighbour;
      if (lane == 0) {
        if (nn >= 0) atomicAdd(&L.rc[nn], 1);
        L.nn[a] = nn;
        L.nlo[a] = lo;
        L.nhi[a] = hi;
        set_key_large(L, X, a);
        nnka = (nn < 0 ? kNoNeighbour : nn) | (L.pair[a] != 0 ? (int)kPairBit : 0);
      }
      FJG_PH(const long long q4 = clock64(); if (lane == 0) ph_ra += q4 - q3;)
      named_sync(3, 64);  // warp 1's parts are in S.part
      if (lane == 0) L.tsum[ta] = merge_skipped(S.part, a, L.klo[a], L.khi[a], nnka);
      FJG_PH(if (lane == 0) ph_sa += clock64() - q4;)
    }
    if (!pair || warp >= 2) {
      const int w0 = pair ? 2 : 0;  // warps taking part: w0 .. W-1
      if (nd > kMaxDirty) {
        for (int t = warp - w0; t < S.nt; t += W - w0)
          if (t != ta) tile_summary(L, t);
      } else {
        for (int k = warp - w0; k < nd; k += W - w0)
          if (S.dirty[k] != ta) tile_summary(L, S.dirty[k]);
      }
    }
    FJG_PH(if (warp == 1 && lane == 0) ph_so += clock64() - q5;)
    __syncthreads();  // B4
    FJG_PH(ph_s3c += clock64() - ph4;)
    if (nd > kMaxDirty) {
      for (int k = tid; k < kMaxTiles / 32; k += T) S.dirty_bits[k] = 0;
    } else {
      for (int k = tid; k < nd; k += T) S.dirty_bits[S.dirty[k] >> 5] = 0;
    }
    if (tid == 0) {
      S.n_rescan = 0;
      S.n_dirty = 0;
      S.win_next = 0;
    }
    // the next reads of dirty_bits, n_rescan, n_dirty and win_next follow B1 and B2
  }

  // ---- epilogue: jet count, and constituent ownership from the union-find
  // parents (owner[label] = parent label, or -(jet+1) once promoted)
  __syncthreads();
  if (tid == 0) A.n_jets[e] = S.ctl_njets;
  FJG_PH(if (A.phase) {
    if (tid == 0) {
      atomicAdd(A.phase + kPhTRebuild, (unsigned long long)ph_rb);
      atomicAdd(A.phase + kPhTS1, (unsigned long long)ph_s1);
      atomicAdd(A.phase + kPhTS2, (unsigned long long)ph_s2);
      atomicAdd(A.phase + kPhTS3a, (unsigned long long)ph_s3a);
      atomicAdd(A.phase + kPhTS3b, (unsigned long long)ph_s3b);
      atomicAdd(A.phase + kPhTS3c, (unsigned long long)ph_s3c);
      atomicAdd(A.phase + kPhTSteps, (unsigned long long)step);
      atomicAdd(A.phase + kPhTEvents, 1ull);
      atomicAdd(A.phase + kPhTTargets, (unsigned long long)ph_tg);
      atomicAdd(A.phase + kPhTTargetSteps, (unsigned long long)ph_tgs);
    }
    if (warp == 1 && lane == 0) atomicAdd(A.phase + kPhTKin, (unsigned long long)ph_kin);
    if (tid == 32 * MW) atomicAdd(A.phase + kPhTDetect, (unsigned long long)ph_det);
    if (tid == 0) {
      atomicAdd(A.phase + kPhTListUpd, (unsigned long long)ph_lu);
      atomicAdd(A.phase + kPhTWindowT0, (unsigned long long)ph_wp);
      atomicAdd(A.phase + kPhTResolveA, (unsigned long long)ph_ra);
      atomicAdd(A.phase + kPhTSumA, (unsigned long long)ph_sa);
    }
    if (warp == 1 && lane == 0) {
      atomicAdd(A.phase + kPhTTargetsW1, (unsigned long long)ph_tt);
      atomicAdd(A.phase + kPhTSumW1, (unsigned long long)ph_so);
    }
  })
  if (A.owner) {
    for (int s = tid; s < N; s += T) {
      int x = s, guard = 0;
      int v = A.owner[off + x];
      while (v >= 0 && v != x && guard < N) {
        x = v;
        v = A.owner[off + x];
        ++guard;
      }
      L.pos[s] = (v < 0) ? (-v - 1) : -1;
    }
    __syncthreads();
    for (int s = tid; s < N; s += T) A.owner[off + s] = L.pos[s];
  }
  __syncthreads();
}

}  // namespace fjg
