// SELL-32x4 layout and the per-lane row kernels shared by the single-system
// solvers (sell.cu) and the batched solver (batch.cu).
//
// Slices of 32 rows (one warp); entry k of the row of lane `lane` sits at
// sell_pos(lane, k) inside its slice: packs of 4 consecutive entries per lane,
// lanes interleaved pack by pack, so that every pack of a warp is one
// contiguous run and each lane loads its 4 entries with a single 16-byte load.
#pragma once

#include "fgb_common.cuh"

namespace fgb {

constexpr int kSellC = 32;        // rows per slice (one warp)
constexpr int kSellPack = 4;      // consecutive entries of a row stored contiguously
constexpr int kSellWindow = 256;  // rows sorted together

// Offset of entry k of lane (row slot) `lane` inside its slice: packs of 4
// entries per lane, lanes interleaved pack by pack, so that pack q of the
// warp is one contiguous 512-byte (FP32) run and each lane loads its 4
// entries with a single 16-byte vector load.
__host__ __device__ __forceinline__ int64_t sell_pos(int lane, int k) {
  return static_cast<int64_t>(k >> 2) * (kSellC * kSellPack) + lane * kSellPack + (k & 3);
}

// One pack (4 entries of this lane's row): 16-byte streaming loads of the
// columns and values, then the gathers.
struct Pack4F {
  int4 c;
  float4 v;
};
struct Pack4D {
  int4 c;
  double2 v01, v23;
};

__device__ __forceinline__ Pack4F load_pack(const int32_t* col, const float* val, int64_t sbase, int lane, int q) {
  const int64_t off = sbase + static_cast<int64_t>(q) * (kSellC * kSellPack) + lane * kSellPack;
  Pack4F p;
  p.c = __ldcs(reinterpret_cast<const int4*>(col + off));
  p.v = __ldcs(reinterpret_cast<const float4*>(val + off));
  return p;
}

__device__ __forceinline__ Pack4D load_pack(const int32_t* col, const double* val, int64_t sbase, int lane, int q) {
  const int64_t off = sbase + static_cast<int64_t>(q) * (kSellC * kSellPack) + lane * kSellPack;
  Pack4D p;
  p.c = __ldcs(reinterpret_cast<const int4*>(col + off));
  p.v01 = __ldcs(reinterpret_cast<const double2*>(val + off));
  p.v23 = __ldcs(reinterpret_cast<const double2*>(val + off + 2));
  return p;
}

template <typename T, typename G>
__device__ __forceinline__ T pack_dot(const Pack4F& p, const G& g, T acc) {
  acc += p.v.x * g(p.c.x);
  acc += p.v.y * g(p.c.y);
  acc += p.v.z * g(p.c.z);
  acc += p.v.w * g(p.c.w);
  return acc;
}

template <typename T, typename G>
__device__ __forceinline__ T pack_dot(const Pack4D& p, const G& g, T acc) {
  acc += p.v01.x * g(p.c.x);
  acc += p.v01.y * g(p.c.y);
  acc += p.v23.x * g(p.c.z);
  acc += p.v23.y * g(p.c.w);
  return acc;
}

template <typename T> struct PackOf;
template <> struct PackOf<float> { using type = Pack4F; };
template <> struct PackOf<double> { using type = Pack4D; };

// Row of slot `lane` of the slice starting at sbase with width w (a multiple of
// 4): sum over entries, in entry order, of val * g(col).  All loads of a trip
// are issued before its gathers: four packs per trip in FP32 (128 bytes of
// matrix per lane in flight), two in FP64 (96 bytes; four would not fit in
// the 64 registers of a 1024-thread block).
template <typename T> struct PacksPerTrip { static constexpr int value = 2; };
template <> struct PacksPerTrip<float> { static constexpr int value = 4; };

// V: stored value type, T: accumulation type (FP32 values of an FP32-assembled
// matrix are accumulated in FP64 by the reliable update).
template <typename V, typename T, typename G>
__device__ __forceinline__ T sell_row_acc(const int32_t* __restrict__ col, const V* __restrict__ val, int64_t sbase,
                                          int w, int lane, const G& g) {
  using P = typename PackOf<V>::type;
  constexpr int U = PacksPerTrip<V>::value;
  const int nq = w / kSellPack;
  T acc = T(0);
  int q = 0;
  for (; q + U <= nq; q += U) {
    P a[U];
#pragma unroll
    for (int u = 0; u < U; ++u) a[u] = load_pack(col, val, sbase, lane, q + u);
#pragma unroll
    for (int u = 0; u < U; ++u) acc = pack_dot<T>(a[u], g, acc);
  }
  for (; q < nq; ++q) {
    const P a = load_pack(col, val, sbase, lane, q);
    acc = pack_dot<T>(a, g, acc);
  }
  return acc;
}

template <typename T, typename G>
__device__ __forceinline__ T sell_row(const int32_t* __restrict__ col, const T* __restrict__ val, int64_t sbase, int w,
                                      int lane, const G& g) {
  return sell_row_acc<T, T, G>(col, val, sbase, w, lane, g);
}

// ------------------------------------------------ delta-coded column indices
// Columns of a row sorted ascending and stored as 16-bit steps: the column of
// entry k is c0 + d[0] + ... + d[k] (c0 per slot, the row's first column;
// d = 0 for the first entry and for padding, which therefore gathers the
// last real column again, with a zero value).  A step above 65535 is bridged
// by zero-valued entries of step 65535.  2 bytes per entry instead of 4.
struct Pack4FH {
  uint2 d;
  float4 v;
};
struct Pack4DH {
  uint2 d;
  double2 v01, v23;
};

__device__ __forceinline__ Pack4FH load_pack_d16(const uint16_t* d16, const float* val, int64_t sbase, int lane,
                                                 int q) {
  const int64_t off = sbase + static_cast<int64_t>(q) * (kSellC * kSellPack) + lane * kSellPack;
  Pack4FH p;
  p.d = __ldcs(reinterpret_cast<const uint2*>(d16 + off));
  p.v = __ldcs(reinterpret_cast<const float4*>(val + off));
  return p;
}

__device__ __forceinline__ Pack4DH load_pack_d16(const uint16_t* d16, const double* val, int64_t sbase, int lane,
                                                 int q) {
  const int64_t off = sbase + static_cast<int64_t>(q) * (kSellC * kSellPack) + lane * kSellPack;
  Pack4DH p;
  p.d = __ldcs(reinterpret_cast<const uint2*>(d16 + off));
  p.v01 = __ldcs(reinterpret_cast<const double2*>(val + off));
  p.v23 = __ldcs(reinterpret_cast<const double2*>(val + off + 2));
  return p;
}

// Columns of a pack from the column before it: a two-level prefix sum of the
// four steps, so that the gathers do not wait on a chain of four additions.
__device__ __forceinline__ int4 pack_cols_d16(uint2 d, int32_t c) {
  const int32_t d0 = static_cast<int32_t>(d.x & 0xffffu), d1 = static_cast<int32_t>(d.x >> 16);
  const int32_t d2 = static_cast<int32_t>(d.y & 0xffffu), d3 = static_cast<int32_t>(d.y >> 16);
  const int32_t c1 = c + (d0 + d1);
  return make_int4(c + d0, c1, c1 + d2, c1 + (d2 + d3));
}

__device__ __forceinline__ int32_t pack_total_d16(uint2 d) {
  return static_cast<int32_t>((d.x & 0xffffu) + (d.x >> 16) + (d.y & 0xffffu) + (d.y >> 16));
}

template <typename T, typename G>
__device__ __forceinline__ T pack_dot_cols(const Pack4FH& p, int4 cc, const G& g, T acc) {
  acc += p.v.x * g(cc.x);
  acc += p.v.y * g(cc.y);
  acc += p.v.z * g(cc.z);
  acc += p.v.w * g(cc.w);
  return acc;
}

template <typename T, typename G>
__device__ __forceinline__ T pack_dot_cols(const Pack4DH& p, int4 cc, const G& g, T acc) {
  acc += p.v01.x * g(cc.x);
  acc += p.v01.y * g(cc.y);
  acc += p.v23.x * g(cc.z);
  acc += p.v23.y * g(cc.w);
  return acc;
}

template <typename T> struct PackD16Of;
template <> struct PackD16Of<float> { using type = Pack4FH; };
template <> struct PackD16Of<double> { using type = Pack4DH; };

// As sell_row_acc, with delta-coded columns starting from c0.
template <typename V, typename T, typename G>
__device__ __forceinline__ T sell_row_acc_d16(const uint16_t* __restrict__ d16, int32_t c0,
                                              const V* __restrict__ val, int64_t sbase, int w, int lane,
                                              const G& g) {
  using P = typename PackD16Of<V>::type;
  constexpr int U = PacksPerTrip<V>::value;
  const int nq = w / kSellPack;
  T acc = T(0);
  int32_t c = c0;
  int q = 0;
  for (; q + U <= nq; q += U) {
    P a[U];
#pragma unroll
    for (int u = 0; u < U; ++u) a[u] = load_pack_d16(d16, val, sbase, lane, q + u);
    // the column before each pack: one addition per pack on the carried chain
    int32_t base[U];
    base[0] = c;
#pragma unroll
    for (int u = 1; u < U; ++u) base[u] = base[u - 1] + pack_total_d16(a[u - 1].d);
    c = base[U - 1] + pack_total_d16(a[U - 1].d);
#pragma unroll
    for (int u = 0; u < U; ++u) acc = pack_dot_cols<T>(a[u], pack_cols_d16(a[u].d, base[u]), g, acc);
  }
  for (; q < nq; ++q) {
    const P a = load_pack_d16(d16, val, sbase, lane, q);
    acc = pack_dot_cols<T>(a, pack_cols_d16(a.d, c), g, acc);
    c += pack_total_d16(a.d);
  }
  return acc;
}

// ------------------------------------------------ 15-bit column steps
// Columns of a row ascending, in the matrix's own numbering (no renumbering):
// the slot's first column c0, then one 16-bit code per entry.  A code below
// 0x8000 is a step: the entry's column is the previous column plus the code.
// A code 0x8000 | h is a long step: a zero-valued entry that gathers the
// previous column again (already in cache) and moves the running column on by
// h * 32768, so that the next step lands on a column far away (FEALPy's
// numbering puts all vertex dofs before all edge dofs: one long step per row
// for P2).  Padding entries have code 0 and value 0.  6 bytes per FP32 entry
// instead of 8, with the gather locality of the original numbering.
// Advance of one code and the offset its gather takes from the column before
// it: a step t moves by t and gathers the new column; a long step moves by
// t * 32768 and gathers the old one.
__device__ __forceinline__ void d15_code(uint32_t code, int32_t& inc, int32_t& own) {
  const int32_t t = static_cast<int32_t>(code & 0x7fffu);
  const bool lng = (code & 0x8000u) != 0u;
  inc = lng ? (t << 15) : t;
  own = lng ? 0 : t;
}

// Columns of a pack from the column before it (base) and the pack's total
// advance, by prefix sums inside the pack: every pack of a trip is decoded
// independently of the others, and only the four totals chain.
__device__ __forceinline__ int4 pack_cols_d15(uint2 d, int32_t base, int32_t& total) {
  int32_t i0, i1, i2, i3, o0, o1, o2, o3;
  d15_code(d.x & 0xffffu, i0, o0);
  d15_code(d.x >> 16, i1, o1);
  d15_code(d.y & 0xffffu, i2, o2);
  d15_code(d.y >> 16, i3, o3);
  const int32_t s01 = i0 + i1;
  total = s01 + (i2 + i3);
  return make_int4(base + o0, base + (i0 + o1), base + (s01 + o2), base + (s01 + (i2 + o3)));
}

// Packs per trip of the 15-bit kernel: a pack carries 24 bytes per FP32
// entry quad instead of 32, so more packs are kept in flight per warp.
template <typename T> struct PacksPerTripD15 { static constexpr int value = 2; };
template <> struct PacksPerTripD15<float> { static constexpr int value = 6; };

// As sell_row_acc, with 15-bit steps and long steps starting from c0.
template <typename V, typename T, typename G>
__device__ __forceinline__ T sell_row_acc_d15(const uint16_t* __restrict__ d16, int32_t c0,
                                              const V* __restrict__ val, int64_t sbase, int w, int lane,
                                              const G& g) {
  using P = typename PackD16Of<V>::type;
  constexpr int U = PacksPerTripD15<V>::value;
  const int nq = w / kSellPack;
  T acc = T(0);
  int32_t c = c0;
  int q = 0;
  for (; q + U <= nq; q += U) {
    P a[U];
#pragma unroll
    for (int u = 0; u < U; ++u) a[u] = load_pack_d16(d16, val, sbase, lane, q + u);
    int4 cc[U];
    int32_t tot[U];
#pragma unroll
    for (int u = 0; u < U; ++u) cc[u] = pack_cols_d15(a[u].d, 0, tot[u]);
    int32_t base = c;
#pragma unroll
    for (int u = 0; u < U; ++u) {
      const int4 k = make_int4(cc[u].x + base, cc[u].y + base, cc[u].z + base, cc[u].w + base);
      acc = pack_dot_cols<T>(a[u], k, g, acc);
      base += tot[u];
    }
    c = base;
  }
  for (; q < nq; ++q) {
    const P a = load_pack_d16(d16, val, sbase, lane, q);
    int32_t tot;
    const int4 k = pack_cols_d15(a.d, c, tot);
    acc = pack_dot_cols<T>(a, k, g, acc);
    c += tot;
  }
  return acc;
}

// ------------------------------------------------ node triples (vector problems)
// For a vector space with three interleaved components (dof = 3 node + comp)
// every nonzero of a row sits in a run of three consecutive columns 3c..3c+2:
// one 4-byte column per triple (3c) and the triple's three values, zero where
// the matrix has no entry.  FP32: 16 bytes per three entries instead of 24.
// Triple slots follow the same SELL-32x4 layout as scalar entries (four
// triples per lane and pack); the values of slot k are val[3k..3k+2].
struct Tri4F {
  int4 c;
  float4 a, b, d;  // a.x a.y a.z | a.w b.x b.y | b.z b.w d.x | d.y d.z d.w
};
struct Tri4D {
  int4 c;
  double2 v0, v1, v2, v3, v4, v5;
};

__device__ __forceinline__ Tri4F load_triples(const int32_t* col, const float* val, int64_t off) {
  Tri4F t;
  t.c = __ldcs(reinterpret_cast<const int4*>(col + off));
  const float4* v = reinterpret_cast<const float4*>(val + 3 * off);
  t.a = __ldcs(v);
  t.b = __ldcs(v + 1);
  t.d = __ldcs(v + 2);
  return t;
}

__device__ __forceinline__ Tri4D load_triples(const int32_t* col, const double* val, int64_t off) {
  Tri4D t;
  t.c = __ldcs(reinterpret_cast<const int4*>(col + off));
  const double2* v = reinterpret_cast<const double2*>(val + 3 * off);
  t.v0 = __ldcs(v);
  t.v1 = __ldcs(v + 1);
  t.v2 = __ldcs(v + 2);
  t.v3 = __ldcs(v + 3);
  t.v4 = __ldcs(v + 4);
  t.v5 = __ldcs(v + 5);
  return t;
}

template <typename T, typename G>
__device__ __forceinline__ T triple_dot(T acc, int32_t c, T a, T b, T d, const G& g) {
  acc += a * g(c);
  acc += b * g(c + 1);
  acc += d * g(c + 2);
  return acc;
}

template <typename T, typename G>
__device__ __forceinline__ T triples_dot(const Tri4F& t, const G& g, T acc) {
  acc = triple_dot<T>(acc, t.c.x, t.a.x, t.a.y, t.a.z, g);
  acc = triple_dot<T>(acc, t.c.y, t.a.w, t.b.x, t.b.y, g);
  acc = triple_dot<T>(acc, t.c.z, t.b.z, t.b.w, t.d.x, g);
  acc = triple_dot<T>(acc, t.c.w, t.d.y, t.d.z, t.d.w, g);
  return acc;
}

template <typename T, typename G>
__device__ __forceinline__ T triples_dot(const Tri4D& t, const G& g, T acc) {
  acc = triple_dot<T>(acc, t.c.x, t.v0.x, t.v0.y, t.v1.x, g);
  acc = triple_dot<T>(acc, t.c.y, t.v1.y, t.v2.x, t.v2.y, g);
  acc = triple_dot<T>(acc, t.c.z, t.v3.x, t.v3.y, t.v4.x, g);
  acc = triple_dot<T>(acc, t.c.w, t.v4.y, t.v5.x, t.v5.y, g);
  return acc;
}

template <typename T> struct TriplesOf;
template <> struct TriplesOf<float> { using type = Tri4F; static constexpr int trip = 2; };
template <> struct TriplesOf<double> { using type = Tri4D; static constexpr int trip = 1; };

// Row of slot `lane` of a node-triple slice (w triples, a multiple of 4):
// packs of four triples, loaded before their gathers (two packs per trip in
// FP32, one in FP64).
template <typename V, typename T, typename G>
__device__ __forceinline__ T sell_row_acc_b3(const int32_t* __restrict__ col, const V* __restrict__ val,
                                             int64_t sbase, int w, int lane, const G& g) {
  using P = typename TriplesOf<V>::type;
  constexpr int U = TriplesOf<V>::trip;
  const int nq = w / kSellPack;
  T acc = T(0);
  int q = 0;
  for (; q + U <= nq; q += U) {
    P t[U];
#pragma unroll
    for (int u = 0; u < U; ++u)
      t[u] = load_triples(col, val, sbase + static_cast<int64_t>(q + u) * (kSellC * kSellPack) + lane * kSellPack);
#pragma unroll
    for (int u = 0; u < U; ++u) acc = triples_dot<T>(t[u], g, acc);
  }
  for (; q < nq; ++q) {
    const P t = load_triples(col, val, sbase + static_cast<int64_t>(q) * (kSellC * kSellPack) + lane * kSellPack);
    acc = triples_dot<T>(t, g, acc);
  }
  return acc;
}

template <typename T>
struct GatherX {
  const T* __restrict__ x;
  __device__ __forceinline__ T operator()(int32_t j) const { return x[j]; }
};

// Gather through L2 only (ld.global.cg): for vectors that other blocks of the
// same (persistent) kernel rewrite between phases, where an L1 line filled in
// an earlier phase would be stale.
template <typename T>
struct GatherCG {
  const T* x;
  __device__ __forceinline__ T operator()(int32_t j) const { return __ldcg(x + j); }
};

}  // namespace fgb
