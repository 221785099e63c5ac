// Surface-triangle argmin shared by the grid-node contact (fwd.cu) and the rope contact (rope.cu):
// find_closest, fem_sensor.py:344-359 — the first triangle whose centroid distance
// |c - p| (norm with eps 1e-10) is smallest, or -1 when none is below 100.
//
// A sensor's centroids are kept in contact-search order (tri_perm: groups of 32 consecutive
// positions are compact patches of the rest surface), each carrying its original index in .w.  A CTA
// stages them in shared memory with the bounding box of every group.  LPN lanes (eight for grid
// nodes, four for rope particles) share one query point: (1) the group with the nearest box, (2) its
// 32 centroids, (3) every other group whose box is not farther than that distance by more than 1e-5
// relative — far above the few-ulp rounding of either distance, so no skipped member could win or
// tie — all LPN lanes together.
// (distance, original index) pairs are combined lexicographically, which is the sequential scan's
// first-minimum-wins result; every distance is evaluated with separately rounded operations, so the
// argmin is bit-identical to a sequential CPU scan.
#pragma once
#include "common.cuh"

struct Best {
  float d;
  int i;
};
DT_DEV Best lexmin(Best a, Best b) { return (b.d < a.d || (b.d == a.d && b.i < a.i)) ? b : a; }
// lexicographic minimum over the LPN lanes (a power of two) that share one query
template <int LPN>
DT_DEV Best group_min(Best b) {
#pragma unroll
  for (int o = 1; o < LPN; o <<= 1) {
    Best other{__shfl_xor_sync(0xffffffffu, b.d, o), __shfl_xor_sync(0xffffffffu, b.i, o)};
    b = lexmin(b, other);
  }
  return b;
}
// float min / max over the warp through the order-preserving map of IEEE bits to int32
DT_DEV int f2ord(float x) {
  const int i = __float_as_int(x);
  return i >= 0 ? i : i ^ 0x7fffffff;
}
DT_DEV float ord2f(int k) { return __int_as_float(k >= 0 ? k : k ^ 0x7fffffff); }
DT_DEV float ord_min(float x) { return ord2f(__reduce_min_sync(0xffffffffu, f2ord(x))); }
DT_DEV float ord_max(float x) { return ord2f(__reduce_max_sync(0xffffffffu, f2ord(x))); }
// Euclidean distance from p to an axis-aligned box (0 inside)
DT_DEV float box_dist(float4 lo, float4 hi, float px, float py, float pz) {
  const float dx = fmaxf(fmaxf(lo.x - px, px - hi.x), 0.f);
  const float dy = fmaxf(fmaxf(lo.y - py, py - hi.y), 0.f);
  const float dz = fmaxf(fmaxf(lo.z - pz, pz - hi.z), 0.f);
  return sqrtf(dx * dx + dy * dy + dz * dz);
}

// Shared-memory words of the staging area for up to `cap` centroids (centroids + 2 boxes per group).
inline size_t stage_bytes(int cap) { return (size_t)((cap > 0 ? cap : 1) + 2 * ((cap + 31) / 32)) * sizeof(float4); }

// Stage sensor S's centroids and group boxes; every thread of the CTA calls it (barriers inside).
template <int NTH>
DT_DEV void stage_sensor(const dt_world& w, const dt_sensor& S, float4* scent, float4* gbox) {
  const int tid = threadIdx.x, nf = S.nf;
  const float4* cent = reinterpret_cast<const float4*>(w.tri_cent);
  __syncthreads();
  for (int t = tid; t < nf; t += NTH) scent[t] = __ldg(cent + S.f_off + t);
  __syncthreads();
  // one warp per group, min/max over the lanes as order-preserving integer reductions
  const int G = (nf + 31) >> 5;
  for (int gg = tid >> 5; gg < G; gg += NTH / 32) {
    const int t = 32 * gg + (tid & 31);
    const float4 c = scent[t < nf ? t : 32 * gg];
    const float4 lo = make_float4(ord_min(c.x), ord_min(c.y), ord_min(c.z), 0.f);
    const float4 hi = make_float4(ord_max(c.x), ord_max(c.y), ord_max(c.z), 0.f);
    if ((tid & 31) == 0) {
      gbox[2 * gg] = lo;
      gbox[2 * gg + 1] = hi;
    }
  }
  __syncthreads();
}

// Largest and smallest Euclidean distance between two axis-aligned boxes.
DT_DEV float box_box_max(float4 alo, float4 ahi, float4 blo, float4 bhi) {
  const float dx = fmaxf(fabsf(ahi.x - blo.x), fabsf(bhi.x - alo.x));
  const float dy = fmaxf(fabsf(ahi.y - blo.y), fabsf(bhi.y - alo.y));
  const float dz = fmaxf(fabsf(ahi.z - blo.z), fabsf(bhi.z - alo.z));
  return sqrtf(dx * dx + dy * dy + dz * dz);
}
DT_DEV float box_box_min(float4 alo, float4 ahi, float4 blo, float4 bhi) {
  const float dx = fmaxf(fmaxf(blo.x - ahi.x, alo.x - bhi.x), 0.f);
  const float dy = fmaxf(fmaxf(blo.y - ahi.y, alo.y - bhi.y), 0.f);
  const float dz = fmaxf(fmaxf(blo.z - ahi.z, alo.z - bhi.z), 0.f);
  return sqrtf(dx * dx + dy * dy + dz * dz);
}

// Groups that can hold the nearest centroid of any query point inside the box [qlo, qhi] (used for
// sensors of more than 32 groups): every centroid of group g lies within box_box_max(q, g) of every
// query, so no query's nearest centroid is farther than U = min_g box_box_max(q, g), and a group
// whose box is farther than U from the query box (with a 1e-4 relative margin, far above rounding)
// holds neither the nearest centroid nor one tied with it.  Writes the group indices, in no
// particular order, to cand and returns their number; `sh` is 2 ints of shared scratch; every
// thread of the CTA calls it (barriers inside).
template <int NTH>
DT_DEV int block_candidates(const float4* gbox, int G, float4 qlo, float4 qhi, int* cand, int* sh) {
  const int tid = threadIdx.x;
  __syncthreads();  // cand and sh may still be read by the previous query box's search
  if (tid == 0) {
    sh[0] = f2ord(3.4e38f);
    sh[1] = 0;
  }
  __syncthreads();
  float u = 3.4e38f;
  for (int g = tid; g < G; g += NTH) u = fminf(u, box_box_max(qlo, qhi, gbox[2 * g], gbox[2 * g + 1]));
  u = ord_min(u);
  if ((tid & 31) == 0) atomicMin(sh, f2ord(u));
  __syncthreads();
  const float U = ord2f(sh[0]) * (1.f + 1e-4f);
  for (int g = tid; g < G; g += NTH)
    if (!(box_box_min(qlo, qhi, gbox[2 * g], gbox[2 * g + 1]) > U)) cand[atomicAdd(sh + 1, 1)] = g;
  __syncthreads();
  return sh[1];
}

// Argmin for the query point (px, py, pz) shared by LPN consecutive lanes (`sub` = lane index within
// them, LPN in {4, 8}); all 32 lanes of the warp call it, `active` false for lane groups without a
// query.  Returns the local triangle index (original order) or -1, in every lane of the group.
// in_smem: S staged by stage_sensor; otherwise a direct scan of global centroids.  cand / nc: the
// groups to search (block_candidates of a box holding the query), or null for all of them.
template <int LPN>
DT_DEV int closest_tri(const dt_world& w, const dt_sensor& S, const float4* scent, const float4* gbox, bool in_smem,
                       bool active, float px, float py, float pz, int sub, const int* cand = nullptr, int nc = 0) {
  const int nf = S.nf;
  Best bb{100.f, -1};
  if (in_smem) {
    const int Gu = cand ? nc : (nf + 31) >> 5;  // groups searched; warp-uniform trip count around the shuffles
    const int G = active ? Gu : 0;
    auto grp = [&](int c) { return cand ? cand[c] : c; };  // group of search position c
    // up to 32 groups: each lane keeps its groups' box distances (position sub + LPN jj) in
    // registers for the pruning pass; beyond that the pass recomputes them
    constexpr int KM = 32 / LPN;
    const bool cached = Gu <= 32;  // warp-uniform
    float bd[KM];
    Best gbest{3.4e38f, 0x7fffffff};
    if (cached) {
#pragma unroll
      for (int jj = 0; jj < KM; ++jj) {
        const int c = sub + LPN * jj;
        bd[jj] = 3.4e38f;
        if (c < G) {
          const int gg = grp(c);
          bd[jj] = box_dist(gbox[2 * gg], gbox[2 * gg + 1], px, py, pz);
          gbest = lexmin(gbest, Best{bd[jj], gg});
        }
      }
    } else {
      for (int c = sub; c < G; c += LPN) {
        const int gg = grp(c);
        gbest = lexmin(gbest, Best{box_dist(gbox[2 * gg], gbox[2 * gg + 1], px, py, pz), gg});
      }
    }
    gbest = group_min<LPN>(gbest);
    // no group is selected when every box distance is NaN (non-finite sensor positions): the
    // sentinel must not be used as an index; the pruned scan below then covers every group
    const int g0 = gbest.i != 0x7fffffff ? gbest.i : -1;
    if (g0 >= 0) {
#pragma unroll
      for (int jj = 0; jj < 32 / LPN; ++jj) {
        const int t = 32 * g0 + sub + LPN * jj;
        if (t < nf) {
          const float4 c = scent[t];
          bb = lexmin(bb, Best{cent_dist(c, px, py, pz), __float_as_int(c.w)});
        }
      }
    }
    bb = group_min<LPN>(bb);
    const float thr = bb.d * (1.f + 1e-5f);
    for (int gc = 0; gc < Gu; gc += 64) {
      unsigned long long live = 0ull;
      const int ge = min(gc + 64, G);
      if (cached) {
#pragma unroll
        for (int jj = 0; jj < KM; ++jj) {
          const int c = sub + LPN * jj;
          if (c < ge && grp(c) != g0 && !(bd[jj] > thr)) live |= 1ull << c;
        }
      } else {
        for (int c = gc + sub; c < ge; c += LPN) {
          const int gg = grp(c);
          if (gg != g0 && !(box_dist(gbox[2 * gg], gbox[2 * gg + 1], px, py, pz) > thr)) live |= 1ull << (c - gc);
        }
      }
#pragma unroll
      for (int o = 1; o < LPN; o <<= 1) live |= __shfl_xor_sync(0xffffffffu, live, o);
      while (live) {
        const int gg = grp(gc + __ffsll((long long)live) - 1);
        live &= live - 1ull;
#pragma unroll
        for (int jj = 0; jj < 32 / LPN; ++jj) {
          const int t = 32 * gg + sub + LPN * jj;
          if (t < nf) {
            const float4 c = scent[t];
            bb = lexmin(bb, Best{cent_dist(c, px, py, pz), __float_as_int(c.w)});
          }
        }
      }
    }
  } else if (active) {
    const float4* cent = reinterpret_cast<const float4*>(w.tri_cent) + S.f_off;
    for (int t = sub; t < nf; t += LPN) {
      const float4 c = __ldg(cent + t);
      bb = lexmin(bb, Best{cent_dist(c, px, py, pz), __float_as_int(c.w)});
    }
  }
  return group_min<LPN>(bb).i;
}
