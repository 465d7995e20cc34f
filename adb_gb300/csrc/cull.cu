// iAABB culling on the GPU (the reference's IAABB::iaabb_brute_force,
// model/iaabb.cpp:545-568, with the narrow phase of model/thread_local_culling.cpp):
//
//  1. vertex projection x = A xbar + p at q, q + alpha dq, or both (trajectory)
//  2. body boxes: inflated rest box through A (iaabb.cpp:40-72), or the union over the
//     trajectory (vtn 3)
//  3. body overlaps: every pair of one scene whose boxes overlap, as a symmetric CSR
//     (both (I,J) and (J,I)) whose upper entries are the unique overlaps, each with its
//     intersection ("cull") box (iaabb.cpp:98-202)
//  4. binning: the vertices, edges and faces of each side that touch the cull box
//     (iaabb.cpp:315-443)
//  5. narrow phase over the flattened candidate space of all overlaps:
//     (v of I) x (f of J), (v of J) x (f of I), (e of I) x (e of J); AABB test, then the
//     exact distance type and distance < dhat (vtn 1/2) or the CCD root (vtn 3)
//  6. vertex-ground pairs (y + 0.5)^2 < dhat, or the ground time of impact
//
// All stage outputs are produced by count -> scan -> ordered write, so every pair list
// comes out in the same order on every run (overlap, then candidate order). The AABB
// tests first run on float copies of the boxes rounded outward (__double2float_rd/_ru):
// a float miss implies an exact miss, so the float prefilter never changes the result
// and saves the scarce FP64 pipe (GB300: 1.2 TFLOP/s FP64 vs 70 TFLOP/s FP32).
#include "abd_engine.h"
#include "abd_exact.cuh"

namespace abd {

namespace {

__device__ __forceinline__ d3 ldX(const double* X, int nv, int v) { return mk(X[v], X[nv + v], X[2 * nv + v]); }

// ---------------------------------------------------------------------------------
// 1. projection: which 0 -> X0 at q0; 1 -> X and Xq at q; 2 -> X at q + alpha dq;
//    3 -> Xq at q only
// The trial state q + alpha dq of every body (alpha per scene when given), once per body
// rather than once per vertex.
__global__ void k_trial_state(Geo g, double alpha) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= 12 * g.nb) return;
  const int b = i / 12;
  const double a = g.alpha_s ? g.alpha_s[g.bscene[b]] : alpha;
  g.qa[i] = XA(g.q[i], XM(g.dq[i], a));
}

__global__ void k_project(Geo g, int which, double alpha) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= g.nv) return;
  int b = g.vbody[v];
  (void)alpha;
  const double* qq = (which == 0) ? g.q0 + 12 * b : ((which == 2) ? g.qa + 12 * b : g.q + 12 * b);
  d3 x = project(qq, g.rest[3 * v], g.rest[3 * v + 1], g.rest[3 * v + 2]);
  double* dst = (which == 0) ? g.X0 : ((which == 3) ? g.Xq : g.X);
  dst[v] = x.x;
  dst[g.nv + v] = x.y;
  dst[2 * g.nv + v] = x.z;
  if (which == 1) {
    g.Xq[v] = x.x;
    g.Xq[g.nv + v] = x.y;
    g.Xq[2 * g.nv + v] = x.z;
  }
}

// 2. body boxes
__global__ void k_body_boxes(Geo g, int vtn, double alpha, double* bbox, float* fbox) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.nb) return;
  box r{mk(g.rest_box[6 * b], g.rest_box[6 * b + 1], g.rest_box[6 * b + 2]),
        mk(g.rest_box[6 * b + 3], g.rest_box[6 * b + 4], g.rest_box[6 * b + 5])};
  double q[12], qt[12];
  if (vtn == 2 && g.alpha_s) alpha = g.alpha_s[g.bscene[b]];
#pragma unroll
  for (int i = 0; i < 12; ++i) {
    q[i] = g.q[12 * b + i];
    qt[i] = XA(q[i], XM(g.dq[12 * b + i], alpha));
  }
  box o;
  if (vtn == 1) o = affine_box(r, q);
  else if (vtn == 2) o = affine_box(r, qt);
  else o = merge(affine_box(r, q), affine_box(r, qt));
  bbox[6 * b] = o.lo.x; bbox[6 * b + 1] = o.lo.y; bbox[6 * b + 2] = o.lo.z;
  bbox[6 * b + 3] = o.hi.x; bbox[6 * b + 4] = o.hi.y; bbox[6 * b + 5] = o.hi.z;
  // the same box in float, rounded outward: a float miss is an exact miss
  fbox[6 * b] = __double2float_rd(o.lo.x); fbox[6 * b + 1] = __double2float_rd(o.lo.y);
  fbox[6 * b + 2] = __double2float_rd(o.lo.z); fbox[6 * b + 3] = __double2float_ru(o.hi.x);
  fbox[6 * b + 4] = __double2float_ru(o.hi.y); fbox[6 * b + 5] = __double2float_ru(o.hi.z);
}

// Float overlap of body boxes i and j (closed intervals, like intersection()).
__device__ __forceinline__ bool fbox_meet(const float* fb, int i, int j) {
  const float* a = fb + 6 * i;
  const float* b = fb + 6 * j;
  return a[0] <= b[3] && a[3] >= b[0] && a[1] <= b[4] && a[4] >= b[1] && a[2] <= b[5] && a[5] >= b[2];
}

__device__ __forceinline__ box ldbox(const double* bb, int i) {
  return box{mk(bb[6 * i], bb[6 * i + 1], bb[6 * i + 2]), mk(bb[6 * i + 3], bb[6 * i + 4], bb[6 * i + 5])};
}

// 3. overlaps: one warp per body row i, j over its scene (j != i), in increasing j; the
// FP64 intersection runs only where the outward-rounded float boxes meet.
__global__ void k_ov_count(Geo g, const double* bbox, const float* fbb, int* cnt_all, int* cnt_up) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= g.nb) return;
  int i = warp;
  if (!scene_on(g, i)) {
    if (lane == 0) cnt_all[i] = cnt_up[i] = 0;
    return;
  }
  box bi = ldbox(bbox, i);
  int ca = 0, cu = 0;
  for (int j0 = g.scene_beg[i]; j0 < g.scene_end[i]; j0 += 32) {
    int j = j0 + lane;
    bool hit = false;
    if (j < g.scene_end[i] && j != i && fbox_meet(fbb, i, j)) {
      box c;
      hit = intersection(bi, ldbox(bbox, j), c);
    }
    unsigned m = __ballot_sync(0xffffffffu, hit);
    unsigned mu = __ballot_sync(0xffffffffu, hit && j > i);
    ca += __popc(m);
    cu += __popc(mu);
  }
  if (lane == 0) {
    cnt_all[i] = ca;
    cnt_up[i] = cu;
  }
}

__global__ void k_ov_fill(Geo g, const double* bbox, const float* fbb, const int* row_ptr, const int* up_ptr, int* col,
                          int* rowid, int* upidx, int* ovI, int* ovJ, double* ovcull, float* ovcull_f) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= g.nb) return;
  int i = warp;
  if (!scene_on(g, i)) return;
  box bi = ldbox(bbox, i);
  int pa = row_ptr[i], pu = up_ptr[i];
  unsigned below = (1u << lane) - 1u;
  for (int j0 = g.scene_beg[i]; j0 < g.scene_end[i]; j0 += 32) {
    int j = j0 + lane;
    bool hit = false;
    box c;
    if (j < g.scene_end[i] && j != i && fbox_meet(fbb, i, j)) hit = intersection(bi, ldbox(bbox, j), c);
    unsigned m = __ballot_sync(0xffffffffu, hit);
    unsigned mu = __ballot_sync(0xffffffffu, hit && j > i);
    if (hit) {
      int e = pa + __popc(m & below);
      col[e] = j;
      rowid[e] = i;
      if (j > i) {
        int u = pu + __popc(mu & below);
        upidx[e] = u;
        ovI[u] = i;
        ovJ[u] = j;
        double* cb = ovcull + 6 * u;
        cb[0] = c.lo.x; cb[1] = c.lo.y; cb[2] = c.lo.z; cb[3] = c.hi.x; cb[4] = c.hi.y; cb[5] = c.hi.z;
        float* cf = ovcull_f + 6 * u;
        cf[0] = __double2float_rd(c.lo.x); cf[1] = __double2float_rd(c.lo.y); cf[2] = __double2float_rd(c.lo.z);
        cf[3] = __double2float_ru(c.hi.x); cf[4] = __double2float_ru(c.hi.y); cf[5] = __double2float_ru(c.hi.z);
      } else {
        upidx[e] = -1;
      }
    }
    pa += __popc(m);
    pu += __popc(mu);
  }
}

// lower entries (i > j): unique overlap of (j, i) by binary search in row j
__global__ void k_ov_lower(int nnz, const int* row_ptr, const int* col, const int* rowid, int* upidx) {
  int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nnz) return;
  int i = rowid[e], j = col[e];
  if (j > i) return;
  int lo = row_ptr[j], hi = row_ptr[j + 1];
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (col[mid] < i) lo = mid + 1;
    else hi = mid;
  }
  upidx[e] = (lo < row_ptr[j + 1] && col[lo] == i) ? upidx[lo] : -1;
}

// ---------------------------------------------------------------------------------
// Float prefilter boxes of every primitive (outward rounded). Trajectory mode spans the
// positions at q (Xq) and at the target (X).
struct fbox6 {
  float lo[3], hi[3];
};
__device__ __forceinline__ void put_fbox(float* dst, const box& b) {
  dst[0] = __double2float_rd(b.lo.x); dst[1] = __double2float_rd(b.lo.y); dst[2] = __double2float_rd(b.lo.z);
  dst[3] = __double2float_ru(b.hi.x); dst[4] = __double2float_ru(b.hi.y); dst[5] = __double2float_ru(b.hi.z);
}
// Float boxes of the primitives (outward rounded). Vertices first, from their FP64
// positions (at X, or the trajectory from Xq to X); edges and faces are then the float
// unions of their vertices' boxes: rounding down (up) commutes with min (max), so
// rd(min(a, b)) = min(rd a, rd b) and the result equals rounding the FP64 box, without
// any FP64 min/max.
__global__ void k_vert_boxes(Geo g, int traj, float* vb) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= g.nv) return;
  d3 p = ldX(g.X, g.nv, t);
  box b = traj ? box2(p, ldX(g.Xq, g.nv, t)) : box{p, p};
  put_fbox(vb + 6 * t, b);
}
__device__ __forceinline__ void fbox_union(float* o, const float* a, const float* b) {
#pragma unroll
  for (int c = 0; c < 3; ++c) {
    o[c] = fminf(o[c], fminf(a[c], b[c]));
    o[c + 3] = fmaxf(o[c + 3], fmaxf(a[c + 3], b[c + 3]));
  }
}
__global__ void k_prim_boxes(Geo g, const float* vb, float* eb, float* fb) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  float o[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  if (t < g.ne) {
    fbox_union(o, vb + 6 * g.ev[2 * t], vb + 6 * g.ev[2 * t + 1]);
#pragma unroll
    for (int c = 0; c < 6; ++c) eb[6 * t + c] = o[c];
    return;
  }
  t -= g.ne;
  if (t < g.nf) {
    const float* v2 = vb + 6 * g.fv[3 * t + 2];
    fbox_union(o, vb + 6 * g.fv[3 * t], vb + 6 * g.fv[3 * t + 1]);
    fbox_union(o, v2, v2);
#pragma unroll
    for (int c = 0; c < 6; ++c) fb[6 * t + c] = o[c];
  }
}

__device__ __forceinline__ bool f_overlap(const float* a, const float* b) {
  return a[0] <= b[3] && a[3] >= b[0] && a[1] <= b[4] && a[4] >= b[1] && a[2] <= b[5] && a[5] >= b[2];
}

// Exact primitive boxes (same construction as the reference's compute_aabb overloads).
__device__ __forceinline__ box vbox_exact(const Geo& g, int v, int traj) {
  d3 p = ldX(g.X, g.nv, v);
  return traj ? box2(p, ldX(g.Xq, g.nv, v)) : box{p, p};
}
__device__ __forceinline__ box ebox_exact(const Geo& g, int e, int traj) {
  int a = g.ev[2 * e], c = g.ev[2 * e + 1];
  d3 p0 = ldX(g.X, g.nv, a), p1 = ldX(g.X, g.nv, c);
  return traj ? box4(p0, p1, ldX(g.Xq, g.nv, a), ldX(g.Xq, g.nv, c)) : box2(p0, p1);
}
__device__ __forceinline__ box fbox_exact(const Geo& g, int f, int traj) {
  int a = g.fv[3 * f], c = g.fv[3 * f + 1], d = g.fv[3 * f + 2];
  box b = box3(ldX(g.X, g.nv, a), ldX(g.X, g.nv, c), ldX(g.X, g.nv, d));
  if (traj) b = merge(box3(ldX(g.Xq, g.nv, a), ldX(g.Xq, g.nv, c), ldX(g.Xq, g.nv, d)), b);
  return b;
}

// 4. binning: one warp per (overlap, side); kinds per side: vertices, edges, faces.
// list slot k of overlap u: 0 vi, 1 ei, 2 fi, 3 vj, 4 ej, 5 fj.
// Binning passes: BIN_COUNT counts each list, BIN_WRITE writes it at offsets from a scan
// of those counts, BIN_ONCE writes it at offsets sized by the body's primitive counts and
// stores the count (one pass instead of two when that capacity fits).
enum { BIN_COUNT = 0, BIN_WRITE = 1, BIN_ONCE = 2 };

// Capacity of list slot (overlap u, side, kind): the primitive count of that body.
__global__ void k_bin_caps(Geo g, int nov, const int* ovI, const int* ovJ, int* cap) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= 6 * nov) return;
  int u = t / 6, side = (t / 3) & 1, kind = t % 3;
  int body = side ? ovJ[u] : ovI[u];
  const int* o = kind == 0 ? g.v_off : (kind == 1 ? g.e_off : g.f_off);
  cap[t] = o[body + 1] - o[body];
}

__global__ void __launch_bounds__(256, 3) k_bin(Geo g, int nov, int pass, int traj, const int* ovI, const int* ovJ, const double* ovcull,
                      const float* ovcull_f, const float* vb, const float* eb, const float* fb, int* cnt,
                      const int* off, int* lst) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= 2 * nov) return;
  int u = warp >> 1, side = warp & 1;
  int body = side ? ovJ[u] : ovI[u];
  float cf[6], ci[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) cf[k] = ovcull_f[6 * u + k];
  // Float bounds inside the FP64 cull box: cull.lo <= ci[0..2], cull.hi >= ci[3..5]. The
  // float box of a primitive is (rd(lo), ru(hi)) of its FP64 box, so rd(lo) < ci_hi gives
  // lo <= nextup(rd(lo)) <= ci_hi <= cull.hi; a primitive passing that on all six sides
  // overlaps the cull box exactly and needs no FP64 test.
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    ci[k] = nextafterf(cf[k], INFINITY);
    ci[k + 3] = nextafterf(cf[k + 3], -INFINITY);
  }
  box cull{mk(ovcull[6 * u], ovcull[6 * u + 1], ovcull[6 * u + 2]),
           mk(ovcull[6 * u + 3], ovcull[6 * u + 4], ovcull[6 * u + 5])};
  unsigned below = (1u << lane) - 1u;
#pragma unroll 1
  for (int kind = 0; kind < 3; ++kind) {
    int beg, end;
    const float* fbx;
    if (kind == 0) { beg = g.v_off[body]; end = g.v_off[body + 1]; fbx = vb; }
    else if (kind == 1) { beg = g.e_off[body]; end = g.e_off[body + 1]; fbx = eb; }
    else { beg = g.f_off[body]; end = g.f_off[body + 1]; fbx = fb; }
    int slot = u * 6 + side * 3 + kind;
    int c = 0, base = pass != BIN_COUNT ? off[slot] : 0;
    // BIN_R runs of 32 per step: their boxes are loaded before any is tested, so the
    // warp keeps several L2 loads in flight
    constexpr int BIN_R = 4;
    for (int k0 = beg; k0 < end; k0 += 32 * BIN_R) {
      float q[BIN_R][6];
#pragma unroll
      for (int r = 0; r < BIN_R; ++r) {
        const int k = k0 + 32 * r + lane;
        if (k < end) {
          const float2* src = reinterpret_cast<const float2*>(fbx + 6 * (size_t)k);
          float2 a = src[0], b = src[1], d = src[2];
          q[r][0] = a.x; q[r][1] = a.y; q[r][2] = b.x; q[r][3] = b.y; q[r][4] = d.x; q[r][5] = d.y;
        } else {
          q[r][0] = q[r][1] = q[r][2] = INFINITY;  // misses every box
          q[r][3] = q[r][4] = q[r][5] = -INFINITY;
        }
      }
#pragma unroll
      for (int r = 0; r < BIN_R; ++r) {
        const int k = k0 + 32 * r + lane;
        bool hit = false;
        if (f_overlap(cf, q[r])) {
          hit = q[r][0] < ci[3] && q[r][1] < ci[4] && q[r][2] < ci[5] && q[r][3] > ci[0] && q[r][4] > ci[1] &&
                q[r][5] > ci[2];
          if (!hit) {
            box b = (kind == 0) ? vbox_exact(g, k, traj) : (kind == 1 ? ebox_exact(g, k, traj) : fbox_exact(g, k, traj));
            hit = overlaps(cull, b);
          }
        }
        unsigned m = __ballot_sync(0xffffffffu, hit);
        if (pass != BIN_COUNT && hit) lst[base + c + __popc(m & below)] = k - beg;
        c += __popc(m);
      }
    }
    if (pass != BIN_WRITE && lane == 0) cnt[slot] = c;
  }
}

constexpr int NT = 256;     // narrow-phase threads per CTA
constexpr int TILE = 384;   // primitives of one list staged in shared memory (2 x 9 kB)
constexpr int REC_CAP = 2048;  // accepted pairs of one overlap kept in shared memory for sorting
// Box-phase candidates per thread between two exact phases (STEP), and the queue of
// float-box hits they fill (NT * STEP entries). A longer box phase runs the exact phase
// less often; a shorter one leaves shared memory for more CTAs per SM. The result does not
// depend on STEP (accepted pairs are sorted by key before they are written, TOIs are
// min-reduced), so the autotuner picks among these variants by time: pair cull (mode 0)
// 32 / 64 / 96, CCD (mode 2) 24 / 36 / 64; the defaults are the middle ones (measured
// fastest on the pile when the choice was fixed).
constexpr int kNarrowVariants = 3;
constexpr int kNarrowStep[2][kNarrowVariants] = {{32, 64, 96}, {24, 36, 64}};
constexpr int kNarrowDefault = 1;
// dynamic shared memory of k_narrow_scan<MODE, STEP>: boxes, queue, accepted pairs (MODE 0)
// (MODE 0 also stages the vertex ids of the staged primitives: 2 per A entry, 3 per B)
__host__ __device__ constexpr size_t narrow_smem(int mode, int step) {
  return 2 * TILE * 6 * sizeof(float) + (size_t)NT * step * sizeof(unsigned) +
         (mode == 0 ? REC_CAP * (sizeof(unsigned long long) + 1) + 5 * TILE * sizeof(int) : 0);
}

__device__ __forceinline__ void finflate(const float* s, float ds, float* o) {
  o[0] = __fsub_rd(s[0], ds); o[1] = __fsub_rd(s[1], ds); o[2] = __fsub_rd(s[2], ds);
  o[3] = __fadd_ru(s[3], ds); o[4] = __fadd_ru(s[4], ds); o[5] = __fadd_ru(s[5], ds);
}

// Order-preserving key of a double for atomicMin on unsigned 64-bit.
__device__ __forceinline__ unsigned long long dkey(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// Exact narrow-phase test of one candidate at the culled configuration (vtn 1/2):
// returns 0 (no pair) or 1 + distance type. sub 0/1: vertex v (global) of body A vs
// face f (global) of body B; sub 2: edge ea vs edge eb.
// The candidate is given by its four vertex ids: (point, triangle) for sub 0/1, (edge a,
// edge b) for sub 2.
__device__ __forceinline__ int exact_pair_v(const Geo& g, const Params& P, int sub, int v0, int v1, int v2, int v3) {
  int nv = g.nv;
  if (sub < 2) {
    d3 p = ldX(g.X, nv, v0);
    box bv = inflate(box{p, p}, P.d_sqrt);
    d3 t0 = ldX(g.X, nv, v1), t1 = ldX(g.X, nv, v2), t2 = ldX(g.X, nv, v3);
    if (!overlaps(bv, box3(t0, t1, t2))) return 0;
    int ty = pt_type(p, t0, t1, t2);
    return (pt_dist(p, t0, t1, t2, ty) < P.dhat) ? 1 + ty : 0;
  }
  d3 a0 = ldX(g.X, nv, v0), a1 = ldX(g.X, nv, v1);
  d3 b0 = ldX(g.X, nv, v2), b1 = ldX(g.X, nv, v3);
  if (!overlaps(inflate(box2(a0, a1), P.d_sqrt), box2(b0, b1))) return 0;
  int ty = ee_type(a0, a1, b0, b1);
  return (ee_dist(a0, a1, b0, b1, ty) < P.dhat) ? 1 + ty : 0;
}
// Vertex ids of candidate (pa, pb): point pa and face pb (sub 0/1), edges pa and pb (sub 2).
__device__ __forceinline__ void pair_vertex_ids(const Geo& g, int sub, int pa, int pb, int (&v)[4]) {
  if (sub < 2) {
    v[0] = pa; v[1] = g.fv[3 * pb]; v[2] = g.fv[3 * pb + 1]; v[3] = g.fv[3 * pb + 2];
  } else {
    v[0] = g.ev[2 * pa]; v[1] = g.ev[2 * pa + 1]; v[2] = g.ev[2 * pb]; v[3] = g.ev[2 * pb + 1];
  }
}
__device__ __forceinline__ int exact_pair(const Geo& g, const Params& P, int sub, int pa, int pb) {
  int v[4];
  pair_vertex_ids(g, sub, pa, pb, v);
  return exact_pair_v(g, P, sub, v[0], v[1], v[2], v[3]);
}

// ---- FP32 lower bounds of pair distances with tracked rounding errors ----
// A value v carries a bound e on |v - exact|, where "exact" is the same expression in real
// arithmetic on the FP64 positions. Inputs are the lower corners of the vertex float
// boxes (rd(x), |x - rd(x)| <= 2^-23 |x|); every operation adds its rounding (u |v| with
// u = 2^-24, slightly enlarged, plus an underflow term), and the error terms themselves
// are accumulated rounding up. The bounds are therefore rigorous; they let most float-box
// hits be rejected without the FP64 test (GB300 issues FP64 at 1/64 of the FP32 rate).
struct EF {
  float v, e;
};
__device__ __forceinline__ EF ef_in(float x) { return {x, __fadd_ru(__fmul_ru(fabsf(x), 1.2042e-7f), 1e-37f)}; }
__device__ __forceinline__ float ef_rnd(float v) { return __fadd_ru(__fmul_ru(fabsf(v), 6.0e-8f), 1e-37f); }
__device__ __forceinline__ EF ef_add(EF a, EF b) {
  const float v = __fadd_rn(a.v, b.v);
  return {v, __fadd_ru(__fadd_ru(a.e, b.e), ef_rnd(v))};
}
__device__ __forceinline__ EF ef_sub(EF a, EF b) {
  const float v = __fsub_rn(a.v, b.v);
  return {v, __fadd_ru(__fadd_ru(a.e, b.e), ef_rnd(v))};
}
__device__ __forceinline__ EF ef_mul(EF a, EF b) {
  const float v = __fmul_rn(a.v, b.v);
  float e = __fadd_ru(__fmul_ru(fabsf(a.v), b.e), __fmul_ru(fabsf(b.v), a.e));
  e = __fadd_ru(e, __fmul_ru(a.e, b.e));
  return {v, __fadd_ru(e, ef_rnd(v))};
}
struct EF3 {
  EF x[3];
};
__device__ __forceinline__ EF3 ef3_in(const float* p) { return {{ef_in(p[0]), ef_in(p[1]), ef_in(p[2])}}; }
__device__ __forceinline__ EF3 ef3_sub(const EF3& a, const EF3& b) {
  return {{ef_sub(a.x[0], b.x[0]), ef_sub(a.x[1], b.x[1]), ef_sub(a.x[2], b.x[2])}};
}
__device__ __forceinline__ EF3 ef3_cross(const EF3& a, const EF3& b) {
  return {{ef_sub(ef_mul(a.x[1], b.x[2]), ef_mul(a.x[2], b.x[1])),
           ef_sub(ef_mul(a.x[2], b.x[0]), ef_mul(a.x[0], b.x[2])),
           ef_sub(ef_mul(a.x[0], b.x[1]), ef_mul(a.x[1], b.x[0]))}};
}
__device__ __forceinline__ EF ef3_dot(const EF3& a, const EF3& b) {
  return ef_add(ef_add(ef_mul(a.x[0], b.x[0]), ef_mul(a.x[1], b.x[1])), ef_mul(a.x[2], b.x[2]));
}
// lower bound of num^2 / den for num known positive by at least lo > 0, den <= den.v + den.e
__device__ __forceinline__ float ef_ratio_lb(float lo, EF den) {
  return __fdiv_rd(__fmul_rd(lo, lo), __fadd_ru(den.v, den.e));
}
// lower bound of |x| (0 when the sign is not certain)
__device__ __forceinline__ float ef_abs_lb(EF x) { return fmaxf(__fsub_rd(fabsf(x.v), x.e), 0.f); }

// Lower bound of the squared point-triangle distance: the point-plane distance combined
// with the largest distance of the point beyond one of the triangle's edge lines in the
// plane (the two components are orthogonal).
__device__ __forceinline__ float lb2_pt_f(const float* p, const float* t0, const float* t1, const float* t2) {
  const EF3 P = ef3_in(p), T0 = ef3_in(t0), T1 = ef3_in(t1), T2 = ef3_in(t2);
  const EF3 e1 = ef3_sub(T1, T0), e2 = ef3_sub(T2, T0), e3 = ef3_sub(T2, T1), w = ef3_sub(P, T0);
  const EF3 n = ef3_cross(e1, e2);
  const EF nn = ef3_dot(n, n);
  const float sl = ef_abs_lb(ef3_dot(w, n));
  float lb = sl > 0.f ? ef_ratio_lb(sl, nn) : 0.f;
  // outward in-plane edge normals m = edge x n (edges t0->t1, t1->t2, t2->t0)
  const EF3 me[3] = {ef3_cross(e1, n), ef3_cross(e3, n), ef3_cross(ef3_sub(T0, T2), n)};
  const EF3 ve[3] = {w, ef3_sub(P, T1), ef3_sub(P, T2)};
  float side = 0.f;
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const EF num = ef3_dot(ve[k], me[k]);
    const float lo = __fsub_rd(num.v, num.e);
    if (lo > 0.f) side = fmaxf(side, ef_ratio_lb(lo, ef3_dot(me[k], me[k])));
  }
  return __fadd_rd(lb, side);
}

// Lower bound of the squared segment-segment distance: the line-line distance combined
// with one in-plane separation: one segment entirely on one side of the other's line, or
// beyond one of its ends along its direction.
__device__ __forceinline__ float lb2_ee_f(const float* a0, const float* a1, const float* b0, const float* b1) {
  const EF3 A0 = ef3_in(a0), A1 = ef3_in(a1), B0 = ef3_in(b0), B1 = ef3_in(b1);
  const EF3 u = ef3_sub(A1, A0), v = ef3_sub(B1, B0);
  const EF3 n = ef3_cross(u, v);
  const EF nn = ef3_dot(n, n);
  const float sl = ef_abs_lb(ef3_dot(ef3_sub(B0, A0), n));
  float lb = sl > 0.f ? ef_ratio_lb(sl, nn) : 0.f;
  float sep = 0.f;
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const EF3& d = k == 0 ? u : v;
    const EF3& base = k == 0 ? A0 : B0;
    const EF3 q0 = ef3_sub(k == 0 ? B0 : A0, base), q1 = ef3_sub(k == 0 ? B1 : A1, base);
    // the other segment on one side of this one's line (in-plane normal n x d)
    const EF3 m = ef3_cross(n, d);
    const EF x0 = ef3_dot(q0, m), x1 = ef3_dot(q1, m);
    float lo = 0.f;
    if (__fsub_rd(x0.v, x0.e) > 0.f && __fsub_rd(x1.v, x1.e) > 0.f)
      lo = fminf(__fsub_rd(x0.v, x0.e), __fsub_rd(x1.v, x1.e));
    else if (__fadd_ru(x0.v, x0.e) < 0.f && __fadd_ru(x1.v, x1.e) < 0.f)
      lo = fminf(-__fadd_ru(x0.v, x0.e), -__fadd_ru(x1.v, x1.e));
    if (lo > 0.f) sep = fmaxf(sep, ef_ratio_lb(lo, ef3_dot(m, m)));
    // the other segment beyond one end of this one along d
    const EF dd = ef3_dot(d, d);
    const EF y0 = ef3_dot(q0, d), y1 = ef3_dot(q1, d);
    const EF z0 = ef_sub(y0, dd), z1 = ef_sub(y1, dd);
    lo = 0.f;
    if (__fsub_rd(z0.v, z0.e) > 0.f && __fsub_rd(z1.v, z1.e) > 0.f)
      lo = fminf(__fsub_rd(z0.v, z0.e), __fsub_rd(z1.v, z1.e));
    else if (__fadd_ru(y0.v, y0.e) < 0.f && __fadd_ru(y1.v, y1.e) < 0.f)
      lo = fminf(-__fadd_ru(y0.v, y0.e), -__fadd_ru(y1.v, y1.e));
    if (lo > 0.f) sep = fmaxf(sep, ef_ratio_lb(lo, dd));
  }
  return __fadd_rd(lb, sep);
}

// Rejects a float-box hit when the float lower bound of its squared distance reaches
// dhat (1 + 1e-4) and the primitives are well shaped (no edge with squared length below
// 2e-6 dhat, no triangle or edge pair with |n|^2 below 2e-6 of the product of the squared
// edge lengths, so the FP64 distance formulas are accurate far inside the 1e-4 margin):
// such a pair is one the FP64 test rejects too, so it never reaches that test.
// The candidate is given by its four vertex ids, as for exact_pair_v.
__device__ __forceinline__ bool f_reject_v(const float* vb, int sub, int v0, int v1, int v2, int v3, float lim) {
  const float *x0 = vb + 6 * v0, *x1 = vb + 6 * v1, *x2 = vb + 6 * v2, *x3 = vb + 6 * v3;
  // well-shaped guards in plain float with twice the FP64 guards' margins
  float ea[3], eb[3];
  for (int c = 0; c < 3; ++c) {
    ea[c] = sub < 2 ? x2[c] - x1[c] : x1[c] - x0[c];
    eb[c] = sub < 2 ? x3[c] - x1[c] : x3[c] - x2[c];
  }
  const float la = ea[0] * ea[0] + ea[1] * ea[1] + ea[2] * ea[2];
  const float lb = eb[0] * eb[0] + eb[1] * eb[1] + eb[2] * eb[2];
  const float nx = ea[1] * eb[2] - ea[2] * eb[1], ny = ea[2] * eb[0] - ea[0] * eb[2], nz = ea[0] * eb[1] - ea[1] * eb[0];
  const float nn = nx * nx + ny * ny + nz * nz;
  float lmin = fminf(la, lb);
  if (sub < 2) {
    const float d0 = x3[0] - x2[0], d1 = x3[1] - x2[1], d2 = x3[2] - x2[2];
    lmin = fminf(lmin, d0 * d0 + d1 * d1 + d2 * d2);
  }
  if (!(lmin >= 2e-6f * lim) || !(nn >= 2e-6f * la * lb)) return false;
  const float l2 = sub < 2 ? lb2_pt_f(x0, x1, x2, x3) : lb2_ee_f(x0, x1, x2, x3);
  return l2 >= lim;
}

// Trajectory time of impact of one candidate (vtn 3), exact box test included.
__device__ __forceinline__ double exact_toi(const Geo& g, int sub, int pa, int pb) {
  int nv = g.nv;
  if (sub < 2) {
    d3 v1 = ldX(g.X, nv, pa), v0 = ldX(g.Xq, nv, pa);
    int i0 = g.fv[3 * pb], i1 = g.fv[3 * pb + 1], i2 = g.fv[3 * pb + 2];
    d3 f1[3] = {ldX(g.X, nv, i0), ldX(g.X, nv, i1), ldX(g.X, nv, i2)};
    d3 f0[3] = {ldX(g.Xq, nv, i0), ldX(g.Xq, nv, i1), ldX(g.Xq, nv, i2)};
    if (!overlaps(box2(v0, v1), merge(box3(f0[0], f0[1], f0[2]), box3(f1[0], f1[1], f1[2])))) return 1.0;
    return pt_collision_time(v0, f0, v1, f1);
  }
  int a0 = g.ev[2 * pa], a1 = g.ev[2 * pa + 1], b0 = g.ev[2 * pb], b1 = g.ev[2 * pb + 1];
  d3 A1[2] = {ldX(g.X, nv, a0), ldX(g.X, nv, a1)}, A0[2] = {ldX(g.Xq, nv, a0), ldX(g.Xq, nv, a1)};
  d3 B1[2] = {ldX(g.X, nv, b0), ldX(g.X, nv, b1)}, B0[2] = {ldX(g.Xq, nv, b0), ldX(g.Xq, nv, b1)};
  if (!overlaps(box4(A0[0], A0[1], A1[0], A1[1]), box4(B0[0], B0[1], B1[0], B1[1]))) return 1.0;
  return ee_collision_time(A0, B0, A1, B1);
}

struct NarrowOut {
  int *pt, *pt_ov, *ee, *ee_ov;
  int8_t *pt_ty, *ee_ty;
};

struct SubLists {
  int A, B, nA, nB, offA, offB;
  const int *LA, *LB;
  const float *boxA, *boxB;
};

__device__ __forceinline__ SubLists sub_lists(const Geo& g, int sub, int I, int J, const int* n, const int* o,
                                              const int* lst, const float* vb, const float* eb, const float* fb) {
  SubLists L;
  int la = sub == 0 ? 0 : (sub == 1 ? 3 : 1);  // vi / vj / ei
  int lb = sub == 0 ? 5 : (sub == 1 ? 2 : 4);  // fj / fi / ej
  L.A = (sub == 1) ? J : I;
  L.B = (sub == 1) ? I : J;
  L.nA = n[la];
  L.nB = n[lb];
  L.boxA = sub < 2 ? vb : eb;
  L.boxB = sub < 2 ? fb : eb;
  L.offA = sub < 2 ? g.v_off[L.A] : g.e_off[L.A];
  L.offB = sub < 2 ? g.f_off[L.B] : g.e_off[L.B];
  L.LA = lst + o[la];
  L.LB = lst + o[lb];
  return L;
}

// Warp-wide union of float boxes (min of lo, max of hi); every lane gets it.
__device__ __forceinline__ void warp_box_union(float* b) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      float v = __shfl_xor_sync(0xffffffffu, b[c], o);
      b[c] = c < 3 ? fminf(b[c], v) : fmaxf(b[c], v);
    }
}

// Keeps, in order and in place, the entries of list L[0..n) whose float box (inflated by
// ds when `infl`) hits box `q`; returns the new length. Each chunk of 32 entries is read
// before any of it is written, and writes never pass reads.
__device__ __forceinline__ int warp_compact(int* L, int n, int off, const float* boxes, bool infl, float ds,
                                            const float* q) {
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  int kept = 0;
  for (int k0 = 0; k0 < n; k0 += 32) {
    int k = k0 + lane;
    int id = 0;
    bool keep = false;
    if (k < n) {
      id = L[k];
      float bx[6];
      const float* src = boxes + 6 * (off + id);
      if (infl) finflate(src, ds, bx);
      else
#pragma unroll
        for (int c = 0; c < 6; ++c) bx[c] = src[c];
      keep = f_overlap(bx, q);
    }
    unsigned m = __ballot_sync(0xffffffffu, keep);
    if (keep) L[kept + __popc(m & below)] = id;
    kept += __popc(m);
  }
  return kept;
}

// 4b. Shrinks the two lists of every sub-problem (one warp per overlap and sub-problem) so
// that every candidate pair whose float boxes hit survives: A keeps the entries hitting
// the union of the B boxes, then B keeps the entries hitting the union of the kept A boxes
// (A inflated by ds for the pair cull, not for trajectories). The reference's loose body
// boxes bin whole caps of both bodies; this leaves the part near the other body, and most
// sub-problems of a pile end up empty before any CTA of the narrow phase is spent on them.
template <bool INFL>
__global__ void k_refine(Geo g, float ds, int nov, const int* ovI, const int* ovJ, int* cnt, const int* off, int* lst,
                         const float* vb, const float* eb, const float* fb) {
  const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= 3 * nov) return;
  const int u = warp / 3, sub = warp - 3 * u;
  int* n = cnt + 6 * u;
  SubLists L = sub_lists(g, sub, ovI[u], ovJ[u], n, off + 6 * u, lst, vb, eb, fb);
  if (L.nA == 0 || L.nB == 0) return;
  float bb[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int k = lane; k < L.nB; k += 32) {
    const float* b = L.boxB + 6 * (L.offB + L.LB[k]);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      bb[c] = fminf(bb[c], b[c]);
      bb[c + 3] = fmaxf(bb[c + 3], b[c + 3]);
    }
  }
  warp_box_union(bb);
  int* LA = const_cast<int*>(L.LA);
  int* LB = const_cast<int*>(L.LB);
  const int nA = warp_compact(LA, L.nA, L.offA, L.boxA, INFL, ds, bb);
  float ba[6] = {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY, -INFINITY};
  for (int k = lane; k < nA; k += 32) {
    float a[6];
    const float* src = L.boxA + 6 * (L.offA + LA[k]);
    if (INFL) finflate(src, ds, a);
    else
#pragma unroll
      for (int c = 0; c < 6; ++c) a[c] = src[c];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
      ba[c] = fminf(ba[c], a[c]);
      ba[c + 3] = fmaxf(ba[c + 3], a[c + 3]);
    }
  }
  warp_box_union(ba);
  const int nB = nA ? warp_compact(LB, L.nB, L.offB, L.boxB, false, ds, ba) : 0;
  if (lane == 0) {
    const int la = sub == 0 ? 0 : (sub == 1 ? 3 : 1), lb = sub == 0 ? 5 : (sub == 1 ? 2 : 4);
    n[la] = nA;
    n[lb] = nB;
  }
}

// Stages one chunk of each list's float boxes in shared memory (A side inflated by
// sqrt(dhat), rounded outward, unless `traj`).
// With sVA / sVB (pair cull) it also stages the vertex ids of the chunk's primitives:
// A entry k at sVA[2k] (a point: its id; an edge: its two), B entry k at sVB[3k] (a face:
// its three; an edge: its two), so the exact phase reads them from shared memory.
__device__ __forceinline__ void stage(const Geo& g, int sub, const SubLists& L, int a0, int ca, int b0, int cb,
                                      bool inflate_a, float ds_f, float* sA, float* sB, int* sVA, int* sVB) {
  __syncthreads();
  for (int k = threadIdx.x; k < ca; k += blockDim.x) {
    const int pa = L.offA + L.LA[a0 + k];
    const float* src = L.boxA + 6 * pa;
    if (inflate_a) finflate(src, ds_f, sA + 6 * k);
    else
#pragma unroll
      for (int c = 0; c < 6; ++c) sA[6 * k + c] = src[c];
    if (sVA) {
      if (sub < 2) {
        sVA[2 * k] = pa;
      } else {
        sVA[2 * k] = g.ev[2 * pa];
        sVA[2 * k + 1] = g.ev[2 * pa + 1];
      }
    }
  }
  for (int k = threadIdx.x; k < cb; k += blockDim.x) {
    const int pb = L.offB + L.LB[b0 + k];
    const float* src = L.boxB + 6 * pb;
#pragma unroll
    for (int c = 0; c < 6; ++c) sB[6 * k + c] = src[c];
    if (sVB) {
      if (sub < 2) {
        sVB[3 * k] = g.fv[3 * pb];
        sVB[3 * k + 1] = g.fv[3 * pb + 1];
        sVB[3 * k + 2] = g.fv[3 * pb + 2];
      } else {
        sVB[3 * k] = g.ev[2 * pb];
        sVB[3 * k + 1] = g.ev[2 * pb + 1];
      }
    }
  }
  __syncthreads();
}

__device__ __forceinline__ bool f_hit(const float* a, const float* b) {
  return a[0] <= b[3] && a[3] >= b[0] && a[1] <= b[4] && a[4] >= b[1] && a[2] <= b[5] && a[5] >= b[2];
}

// Order in which the narrow-phase CTAs take the overlaps: the heaviest sub-problem sets
// first (after refinement a pile's work sits in ~1700 of ~10000 overlaps, from 1k to 56k
// candidate pairs each), so the long ones do not start in the last wave. The outputs of
// an overlap do not depend on when it is processed.
constexpr int NBUCKET = 4;
__device__ __forceinline__ int work_bucket(const int* n) {
  long long c = (long long)n[0] * n[5] + (long long)n[3] * n[2] + (long long)n[1] * n[4];
  return c >= 16384 ? 0 : (c >= 2048 ? 1 : (c > 0 ? 2 : 3));
}
__global__ void k_order_count(int nov, const int* cnt, int* bc) {
  int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u < nov) atomicAdd(&bc[work_bucket(cnt + 6 * u)], 1);
}
__global__ void k_order_place(int nov, const int* cnt, int* bc, int* order) {
  int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nov) return;
  int b = work_bucket(cnt + 6 * u);
  int base = 0;
  for (int k = 0; k < b; ++k) base += bc[k];
  order[base + atomicAdd(&bc[NBUCKET + b], 1)] = u;
}

// 5a. Narrow phase, one CTA per overlap, count (MODE 0) or trajectory TOI (MODE 2).
// For each sub-problem (v(I) x f(J), v(J) x f(I), e(I) x e(J)) the float boxes of both
// lists are staged in shared memory. The work alternates between two phases so that the
// FP64 work is spread evenly over the CTA:
//  - box phase: each thread keeps one A box in registers and walks its B boxes (a
//    shared-memory broadcast per step), STEP candidates per thread, and appends the
//    float-box hits to a shared queue (warp-aggregated);
//  - exact phase: the whole CTA takes the queued candidates round-robin for the exact
//    FP64 test (MODE 0: box, lower bounds, type and distance; MODE 2: time of impact).
template <int MODE, int STEP>
__global__ void __launch_bounds__(NT, (MODE == 2 && STEP <= 36) ? 3 : 2) k_narrow_scan(Geo g, Params P, float ds_f, const int* ovI, const int* ovJ,
                                                    int* cnt, const int* off, int* lst, const float* vb,
                                                    const float* eb, const float* fb, int* sub_cnt,
                                                    unsigned long long* toi_key, unsigned long long* stage_key,
                                                    int8_t* stage_ty, int* stage_off, int* stage_total,
                                                    int stage_cap, const int* order) {
  extern __shared__ __align__(16) unsigned char smem_dyn[];
  unsigned long long* recK = reinterpret_cast<unsigned long long*>(smem_dyn);  // REC_CAP (MODE 0)
  float* sA = reinterpret_cast<float*>(smem_dyn + (MODE == 0 ? REC_CAP * sizeof(unsigned long long) : 0));
  float* sB = sA + TILE * 6;
  unsigned int* sq = reinterpret_cast<unsigned int*>(sB + TILE * 6);
  int8_t* recT = reinterpret_cast<int8_t*>(sq + NT * STEP);
  int* sVA = MODE == 0 ? reinterpret_cast<int*>(recT + REC_CAP) : nullptr;  // 2 * TILE (MODE 0)
  int* sVB = MODE == 0 ? sVA + 2 * TILE : nullptr;                           // 3 * TILE (MODE 0)                         // REC_CAP (MODE 0)
  __shared__ int sq_n[2];
  __shared__ int rec_n, rec_base;
  const int u = order[blockIdx.x];
  const float lim_f = __double2float_ru(P.dhat * (1.0 + 1e-4));
  int* n = cnt + 6 * u;
  const int* o = off + 6 * u;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  int c3s[3] = {0, 0, 0};
  double tmin = 1.0;
  if (threadIdx.x == 0) {
    rec_n = 0;
    sq_n[0] = 0;
    sq_n[1] = 0;
  }
  int par = 0;
#pragma unroll 1
  for (int sub = 0; sub < 3; ++sub) {
    SubLists L = sub_lists(g, sub, ovI[u], ovJ[u], n, o, lst, vb, eb, fb);  // lists refined by k_refine
    if (L.nA == 0 || L.nB == 0) continue;
    int cs = 0;
#pragma unroll 1
    for (int a0 = 0; a0 < L.nA; a0 += TILE) {
      const int ca = min(TILE, L.nA - a0);
#pragma unroll 1
      for (int b0 = 0; b0 < L.nB; b0 += TILE) {
        const int cb = min(TILE, L.nB - b0);
        stage(g, sub, L, a0, ca, b0, cb, MODE != 2, ds_f, sA, sB, sVA, sVB);
        // thread t: rows i = t mod ca (ca < NT) or t, t + NT, ... (ca >= NT); columns
        // j = ph, ph + phases, ... with phases = NT / ca threads sharing a row
        const int rows = ca < NT ? ca : NT;
        const int phases = ca < NT ? NT / ca : 1;
        const int ph = ca < NT ? threadIdx.x / ca : 0;
        const int row0 = threadIdx.x % rows;
        const bool live = ph < phases;
        const int ncol = live ? (cb - ph + phases - 1) / phases : 0;        // columns per row
        const int nrow = (live && ncol > 0) ? (ca - row0 + rows - 1) / rows : 0;  // rows of this thread
        const int max_items = (ca < NT ? 1 : (ca + NT - 1) / NT) * ((cb + phases - 1) / phases);
        const int steps = (max_items + STEP - 1) / STEP;
        int ri = 0, cj = 0;  // cursor: row index (of this thread's rows), column index
        float a[6];
        if (nrow > 0)
#pragma unroll
          for (int c = 0; c < 6; ++c) a[c] = sA[6 * row0 + c];
#pragma unroll 1
        for (int st = 0; st < steps; ++st) {
          // box phase
#pragma unroll 1
          for (int it = 0; it < STEP; ++it) {
            bool hit = false;
            unsigned code = 0;
            if (ri < nrow) {
              int i = row0 + ri * rows, j = ph + cj * phases;
              hit = i < ca && j < cb && f_hit(a, sB + 6 * j);
              code = ((unsigned)i << 16) | (unsigned)j;
              if (++cj == ncol) {
                cj = 0;
                if (++ri < nrow)
#pragma unroll
                  for (int c = 0; c < 6; ++c) a[c] = sA[6 * (row0 + ri * rows) + c];
              }
            }
            unsigned m = __ballot_sync(0xffffffffu, hit);
            if (m) {
              int base = 0;
              if (lane == 0) base = atomicAdd(&sq_n[par], __popc(m));
              base = __shfl_sync(0xffffffffu, base, 0);
              if (hit) sq[base + __popc(m & below)] = code;
            }
          }
          __syncthreads();
          // exact phase
          const int nq = sq_n[par];
          if (threadIdx.x == 0) sq_n[par ^ 1] = 0;
#pragma unroll 1
          for (int k = threadIdx.x; k < nq; k += NT) {
            unsigned code = sq[k];
            int i = (int)(code >> 16), j = (int)(code & 0xffffu);
            if (i >= ca || j >= cb) continue;
            if (MODE == 2) {
              int pa = L.offA + L.LA[a0 + i], pb = L.offB + L.LB[b0 + j];
              tmin = dmin(tmin, exact_toi(g, sub, pa, pb));
            } else {
              const int w0 = sVA[2 * i];
              const int w1 = sub < 2 ? sVB[3 * j] : sVA[2 * i + 1];
              const int w2 = sub < 2 ? sVB[3 * j + 1] : sVB[3 * j];
              const int w3 = sub < 2 ? sVB[3 * j + 2] : sVB[3 * j + 1];
              int f = f_reject_v(vb, sub, w0, w1, w2, w3, lim_f) ? 0 : exact_pair_v(g, P, sub, w0, w1, w2, w3);
              if (f) {
                ++cs;
                int slot = atomicAdd(&rec_n, 1);
                if (slot < REC_CAP) {
                  recK[slot] = ((unsigned long long)sub << 60) | ((unsigned long long)(a0 + i) << 30) |
                               (unsigned long long)(b0 + j);
                  recT[slot] = (int8_t)(f - 1);
                }
              }
            }
          }
          par ^= 1;
          __syncthreads();
        }
      }
    }
    c3s[sub] = cs;
  }
  if (MODE == 0) {
    __shared__ int sh[3][NT / 32];
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      int v = c3s[k];
#pragma unroll
      for (int q = 16; q > 0; q >>= 1) v += __shfl_xor_sync(0xffffffffu, v, q);
      if (lane == 0) sh[k][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
      int t = 0;
      for (int q = 0; q < NT / 32; ++q) t += sh[threadIdx.x][q];
      sub_cnt[3 * u + threadIdx.x] = t;
    }
    // Sort the collected (sub, i, j) keys (bitonic, shared memory) and stage them, so
    // the write pass only copies. Overlaps with more pairs than REC_CAP are marked
    // (stage_off = -1) and written by the recomputing pass instead.
    // stage_total[1] counts the overlaps left to the recomputing pass
    int nr = rec_n;
    if (nr > REC_CAP || nr == 0) {
      if (threadIdx.x == 0) {
        stage_off[u] = (nr == 0) ? 0 : -1;
        if (nr) atomicAdd(stage_total + 1, 1);
      }
      return;
    }
    int np2 = 1;
    while (np2 < nr) np2 <<= 1;
    for (int k = nr + threadIdx.x; k < np2; k += NT) recK[k] = ~0ull;
    __syncthreads();
    for (int size = 2; size <= np2; size <<= 1)
      for (int stride = size >> 1; stride > 0; stride >>= 1) {
        for (int t = threadIdx.x; t < (np2 >> 1); t += NT) {
          int lo = 2 * t - (t & (stride - 1));
          int hi = lo + stride;
          bool up = ((lo & size) == 0);
          unsigned long long a = recK[lo], b = recK[hi];
          if ((a > b) == up) {
            recK[lo] = b;
            recK[hi] = a;
            int8_t ta = recT[lo];
            recT[lo] = recT[hi];
            recT[hi] = ta;
          }
        }
        __syncthreads();
      }
    if (threadIdx.x == 0) {
      int base = atomicAdd(stage_total, nr);
      rec_base = (base + nr <= stage_cap) ? base : -2;
      stage_off[u] = rec_base;
      if (rec_base < 0) atomicAdd(stage_total + 1, 1);
    }
    __syncthreads();
    if (rec_base >= 0)
      for (int k = threadIdx.x; k < nr; k += NT) {
        stage_key[rec_base + k] = recK[k];
        stage_ty[rec_base + k] = recT[k];
      }
  } else {
#pragma unroll
    for (int q = 16; q > 0; q >>= 1) tmin = dmin(tmin, __shfl_xor_sync(0xffffffffu, tmin, q));
    if (lane == 0 && tmin < 1.0) atomicMin(toi_key + 2 * g.bscene[ovI[u]], dkey(tmin));
  }
}

// 5b'. Copy of the staged, sorted pairs of each overlap to their final slots.
__global__ void k_narrow_copy(int nov, const int* ovI, const int* ovJ, const int* off, const int* lst,
                              const int* sub_cnt, const unsigned long long* stage_key, const int8_t* stage_ty,
                              const int* stage_off, const int* ov_pt_off, const int* ov_ee_off, NarrowOut out) {
  int u = blockIdx.x;
  if (u >= nov) return;
  const int* sc = sub_cnt + 3 * u;
  int nr = sc[0] + sc[1] + sc[2];
  int so = stage_off[u];
  if (nr == 0 || so < 0) return;
  int I = ovI[u], J = ovJ[u];
  const int* o = off + 6 * u;
  for (int k = threadIdx.x; k < nr; k += blockDim.x) {
    unsigned long long key = stage_key[so + k];
    int sub = (int)(key >> 60);
    int i = (int)((key >> 30) & 0x3fffffffull), j = (int)(key & 0x3fffffffull);
    int la = sub == 0 ? 0 : (sub == 1 ? 3 : 1), lb = sub == 0 ? 5 : (sub == 1 ? 2 : 4);
    int A = (sub == 1) ? J : I, B = (sub == 1) ? I : J;
    int a_id = lst[o[la] + i], b_id = lst[o[lb] + j];
    if (sub < 2) {
      int idx = ov_pt_off[u] + k;
      out.pt[4 * idx] = A; out.pt[4 * idx + 1] = a_id; out.pt[4 * idx + 2] = B; out.pt[4 * idx + 3] = b_id;
      out.pt_ty[idx] = stage_ty[so + k];
      out.pt_ov[idx] = u;
    } else {
      int idx = ov_ee_off[u] + (k - sc[0] - sc[1]);
      out.ee[4 * idx] = A; out.ee[4 * idx + 1] = a_id; out.ee[4 * idx + 2] = B; out.ee[4 * idx + 3] = b_id;
      out.ee_ty[idx] = stage_ty[so + k];
      out.ee_ov[idx] = u;
    }
  }
}

// 5b. Ordered write for the overlaps whose pairs did not fit the shared-memory sort. The
// (i, j) space of each sub-problem is walked in row-major order (the order of the
// reference's nested loops), NT candidates at a time, with a CTA-wide ordered
// compaction, stopping once the sub-problem's count (from the count pass) is written.
__global__ void __launch_bounds__(NT) k_narrow_write(Geo g, Params P, float ds_f, const int* ovI, const int* ovJ,
                                                     const int* cnt, const int* off, const int* lst, const float* vb,
                                                     const float* eb, const float* fb, const int* sub_cnt,
                                                     const int* ov_pt_off, const int* ov_ee_off, NarrowOut out,
                                                     const int* stage_off) {
  __shared__ int wcnt[NT / 32];
  const int u = blockIdx.x;
  const int* sc = sub_cnt + 3 * u;
  if (sc[0] + sc[1] + sc[2] == 0 || stage_off[u] >= 0) return;
  const int* n = cnt + 6 * u;
  const int* o = off + 6 * u;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned below = (1u << lane) - 1u;
  int run_pt = ov_pt_off[u], run_ee = ov_ee_off[u];
#pragma unroll 1
  for (int sub = 0; sub < 3; ++sub) {
    if (sc[sub] == 0) continue;
    SubLists L = sub_lists(g, sub, ovI[u], ovJ[u], n, o, lst, vb, eb, fb);
    const int need = sc[sub];
    int done = 0;
    const long long tot = (long long)L.nA * L.nB;
#pragma unroll 1
    for (long long k0 = 0; k0 < tot && done < need; k0 += NT) {
      long long k = k0 + threadIdx.x;
      int f = 0, i = 0, j = 0;
      if (k < tot) {
        i = (int)(k / L.nB);
        j = (int)(k - (long long)i * L.nB);
        float a[6];
        finflate(L.boxA + 6 * (L.offA + L.LA[i]), ds_f, a);
        if (f_hit(a, L.boxB + 6 * (L.offB + L.LB[j])))
          f = exact_pair(g, P, sub, L.offA + L.LA[i], L.offB + L.LB[j]);
      }
      unsigned m = __ballot_sync(0xffffffffu, f != 0);
      if (lane == 0) wcnt[w] = __popc(m);
      __syncthreads();
      int pre = 0, total = 0;
#pragma unroll
      for (int q = 0; q < NT / 32; ++q) {
        pre += (q < w) ? wcnt[q] : 0;
        total += wcnt[q];
      }
      if (f) {
        int idx = (sub < 2 ? run_pt : run_ee) + pre + __popc(m & below);
        int* dst = sub < 2 ? out.pt : out.ee;
        dst[4 * idx] = L.A; dst[4 * idx + 1] = L.LA[i]; dst[4 * idx + 2] = L.B; dst[4 * idx + 3] = L.LB[j];
        (sub < 2 ? out.pt_ty : out.ee_ty)[idx] = (int8_t)(f - 1);
        (sub < 2 ? out.pt_ov : out.ee_ov)[idx] = u;
      }
      if (sub < 2) run_pt += total;
      else run_ee += total;
      done += total;
      __syncthreads();
    }
  }
}

__global__ void k_sub_totals(int nov, const int* sub_cnt, int* npt, int* nee) {
  int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nov) return;
  npt[u] = sub_cnt[3 * u] + sub_cnt[3 * u + 1];
  nee[u] = sub_cnt[3 * u + 2];
}

// 6a. vertex-ground pairs: flags + per-CTA counts, then ordered write
__global__ void k_vg_count(Geo g, Params P, int* blk_cnt) {
  __shared__ int sh[32];
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  bool hit = false;
  if (v < g.nv && scene_on(g, g.vbody[v])) {
    double d = XA(g.X[g.nv + v], P.ground_offset);
    d = XM(d, d);
    hit = d < P.dhat;
  }
  unsigned m = __ballot_sync(0xffffffffu, hit);
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = __popc(m);
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
    blk_cnt[blockIdx.x] = s;
  }
}
__global__ void k_vg_write(Geo g, Params P, const int* blk_off, int* vg) {
  __shared__ int sh[32];
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  bool hit = false;
  if (v < g.nv && scene_on(g, g.vbody[v])) {
    double d = XA(g.X[g.nv + v], P.ground_offset);
    d = XM(d, d);
    hit = d < P.dhat;
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned m = __ballot_sync(0xffffffffu, hit);
  if (lane == 0) sh[w] = __popc(m);
  __syncthreads();
  int pre = 0;
  for (int i = 0; i < w; ++i) pre += sh[i];
  if (hit) {
    int idx = blk_off[blockIdx.x] + pre + __popc(m & ((1u << lane) - 1u));
    int b = g.vbody[v];
    vg[2 * idx] = b;
    vg[2 * idx + 1] = v - g.v_off[b];
  }
}
// VG segment per body: first VG pair of body b (pairs are in vertex order)
__global__ void k_vg_seg(int nb, int nvg, const int* vg, int* seg) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b > nb) return;
  int lo = 0, hi = nvg;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (vg[2 * mid] < b) lo = mid + 1;
    else hi = mid;
  }
  seg[b] = lo;
}

// 6b. ground time of impact (collision.cpp:83-105); toi_key points at the ground slot
// of scene 0 (slots alternate pt/ee, ground per scene).
__global__ void k_vg_toi(Geo g, Params P, unsigned long long* toi_key) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= g.nv || !scene_on(g, g.vbody[v])) return;
  double d2 = XA(g.X[g.nv + v], P.ground_offset);
  if (d2 < 0) {
    double d1 = XA(g.Xq[g.nv + v], P.ground_offset);
    double t = XD(d1, XS(d1, d2));
    if (t < 1.0) atomicMin(toi_key + 2 * g.bscene[g.vbody[v]], dkey(t));
  }
}

__global__ void k_fill_u64(unsigned long long* p, int n, unsigned long long v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

// Smallest float >= d (host side).
// Lets the narrow-phase CTAs use more than the default 48 kB of shared memory (once per
// device; the setting is part of this process's context only).
static void narrow_smem_attr() {
  static int done_dev = -1;
  int dev = 0;
  CK(cudaGetDevice(&dev));
  if (done_dev == dev) return;
#define ABD_NARROW_ATTR(M, ST) \
  CK(cudaFuncSetAttribute(k_narrow_scan<M, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)narrow_smem(M, ST)))
  ABD_NARROW_ATTR(0, 32);
  ABD_NARROW_ATTR(0, 64);
  ABD_NARROW_ATTR(0, 96);
  ABD_NARROW_ATTR(2, 24);
  ABD_NARROW_ATTR(2, 36);
  ABD_NARROW_ATTR(2, 64);
#undef ABD_NARROW_ATTR
  done_dev = dev;
}

// Arguments of one narrow-phase launch.
struct NarrowLaunch {
  Geo g;
  Params P;
  float ds_f;
  const int *ovI, *ovJ;
  int* cnt;
  const int* off;
  int* lst;
  const float *vb, *eb, *fb;
  int* sub_cnt;
  unsigned long long *toi_key, *stage_key;
  int8_t* stage_ty;
  int *stage_off, *stage_total;
  int stage_cap;
  const int* order;
};

// k_narrow_scan<mode, kNarrowStep[mode][variant]> over nov overlaps
static void launch_narrow(int mode, int variant, int nov, const NarrowLaunch& a, cudaStream_t s) {
  const int tag = mode == 2 ? K_NARROW_TOI : K_NARROW_SCAN;
#define ABD_NARROW_LAUNCH(M, ST)                                                                                   \
  KLAUNCH(tag, s, k_narrow_scan<M, ST><<<nov, NT, narrow_smem(M, ST), s>>>(                                       \
                      a.g, a.P, a.ds_f, a.ovI, a.ovJ, a.cnt, a.off, a.lst, a.vb, a.eb, a.fb, a.sub_cnt, a.toi_key, \
                      a.stage_key, a.stage_ty, a.stage_off, a.stage_total, a.stage_cap, a.order))
  const int st = kNarrowStep[mode == 2 ? 1 : 0][variant];
  if (mode == 2) {
    if (st == 24) ABD_NARROW_LAUNCH(2, 24);
    else if (st == 36) ABD_NARROW_LAUNCH(2, 36);
    else ABD_NARROW_LAUNCH(2, 64);
  } else {
    if (st == 32) ABD_NARROW_LAUNCH(0, 32);
    else if (st == 64) ABD_NARROW_LAUNCH(0, 64);
    else ABD_NARROW_LAUNCH(0, 96);
  }
#undef ABD_NARROW_LAUNCH
}

// The narrow phase of `mode` (0: pair cull, 1 in the tables: CCD) with the handle's
// chosen variant. The first launch with at least kTuneMinOverlaps overlaps runs every
// variant on the same input, timed with CUDA events, keeps the fastest for the life of
// the handle and leaves the outputs of the last run (all variants give the same outputs;
// `reset`, when given, clears the pair cull's staging counters before each run).
constexpr int kTuneMinOverlaps = 64;
static void narrow_phase(int mode, int nov, const NarrowLaunch& a, CullScratch& cs, int* reset, cudaStream_t s) {
  const int m = mode == 2 ? 1 : 0;
  if (cs.narrow_variant[m] >= 0 || !cs.autotune || nov < kTuneMinOverlaps) {
    launch_narrow(mode, cs.narrow_variant[m] >= 0 ? cs.narrow_variant[m] : kNarrowDefault, nov, a, s);
    return;
  }
  cudaEvent_t ev[kNarrowVariants + 1];
  for (auto& e : ev) CK(cudaEventCreate(&e));
  CK(cudaEventRecord(ev[0], s));
  for (int v = 0; v < kNarrowVariants; ++v) {
    if (reset) CK(cudaMemsetAsync(reset, 0, 2 * sizeof(int), s));
    launch_narrow(mode, v, nov, a, s);
    CK(cudaEventRecord(ev[v + 1], s));
  }
  CK(cudaEventSynchronize(ev[kNarrowVariants]));
  int best = kNarrowDefault;
  for (int v = 0; v < kNarrowVariants; ++v) {
    float t = 0;
    CK(cudaEventElapsedTime(&t, ev[v], ev[v + 1]));
    cs.narrow_ms[m][v] = t;
    if (t < cs.narrow_ms[m][best]) best = v;
  }
  // the default keeps ties and near-ties (within 3%)
  if (!(cs.narrow_ms[m][best] < 0.97f * cs.narrow_ms[m][kNarrowDefault])) best = kNarrowDefault;
  cs.narrow_variant[m] = best;
  for (auto& e : ev) CK(cudaEventDestroy(e));
}


// Fills cs.order with the overlaps heaviest bucket first (k_order_count / k_order_place).
static void order_overlaps(int nov, CullScratch& cs, cudaStream_t s, int tag) {
  cs.order.ensure(nov + 1);
  cs.order_cnt.ensure(2 * NBUCKET);
  CK(cudaMemsetAsync(cs.order_cnt.p, 0, 2 * NBUCKET * sizeof(int), s));
  KLAUNCH(tag, s, k_order_count<<<nblk(nov, 256), 256, 0, s>>>(nov, cs.bin_cnt.p, cs.order_cnt.p));
  KLAUNCH(tag, s, k_order_place<<<nblk(nov, 256), 256, 0, s>>>(nov, cs.bin_cnt.p, cs.order_cnt.p, cs.order.p));
}

float float_round_up(double d) {
  float f = (float)d;
  if ((double)f < d) f = nextafterf(f, INFINITY);
  return f;
}

double key_to_double(unsigned long long k) {
  unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double d;
  memcpy(&d, &b, sizeof(d));
  return d;
}

}  // namespace

int narrow_step_of(int mode, int variant) { return kNarrowStep[mode == 2 ? 1 : 0][variant]; }

void launch_project(const Geo& g, int which, double alpha, cudaStream_t s) {
  if (which == 2 && g.nb > 0) KLAUNCH(K_PROJECT, s, k_trial_state<<<nblk(12ll * g.nb, 256), 256, 0, s>>>(g, alpha));
  if (g.nv == 0) return;
  KLAUNCH(K_PROJECT, s, k_project<<<nblk(g.nv, 256), 256, 0, s>>>(g, which, alpha));
  prof_work(K_PROJECT, g.nv, 48.0 * g.nv);  // rest read + world write per vertex
}

// Narrow phase of a pair cull over binned (and refined, ordered) lists of nov overlaps:
// classification with staging (grown and repeated when it overflows), per-overlap counts
// and offsets, one host read of the totals (pt, ee, vg, staged, unstaged overlaps), then
// the ordered write of the pairs into S.
static void narrow_pairs(const Geo& g, const Params& P, float ds_f, int nov, const int* ovI, const int* ovJ,
                         CullScratch& cs, PairSet& S, int& npt, int& nee, cudaStream_t s) {
  int* d_tot = cs.tmp_int.p;
  cs.blk_a.ensure(nov + 1);
  cs.blk_b.ensure(nov + 1);
  cs.blk_a_off.ensure(nov + 1);
  cs.blk_b_off.ensure(nov + 1);
  cs.sub_cnt.ensure(3 * (size_t)nov + 3);
  cs.stage_off.ensure(nov + 1);
  if (cs.stage_key.cap < (1u << 16)) {
    cs.stage_key.ensure(1u << 16);
    cs.stage_ty.ensure(1u << 16);
  }
  for (int attempt = 0; attempt < 4; ++attempt) {
    CK(cudaMemsetAsync(d_tot + 6, 0, 2 * sizeof(int), s));
    narrow_smem_attr();
    NarrowLaunch a{g, P, ds_f, ovI, ovJ, cs.bin_cnt.p, cs.bin_off.p, cs.lst.p, cs.vbox.p, cs.ebox.p, cs.fbox.p,
                   cs.sub_cnt.p, nullptr, cs.stage_key.p, cs.stage_ty.p, cs.stage_off.p, d_tot + 6,
                   (int)cs.stage_key.cap, cs.order.p};
    narrow_phase(0, nov, a, cs, d_tot + 6, s);
    // per-overlap pair counts and their offsets, read together with the staged total
    KLAUNCH(K_NARROW_WRITE, s, k_sub_totals<<<nblk(nov, 256), 256, 0, s>>>(nov, cs.sub_cnt.p, cs.blk_a.p, cs.blk_b.p));
    scan_exclusive_int(cs.blk_a.p, cs.blk_a_off.p, nov, d_tot + 3, s, cs.vflag_cnt);
    scan_exclusive_int(cs.blk_b.p, cs.blk_b_off.p, nov, d_tot + 4, s, cs.vflag_cnt);
    CK(cudaMemcpyAsync(cs.h_small + 3, d_tot + 3, 5 * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    if ((size_t)cs.h_small[6] <= cs.stage_key.cap) break;
    // staging overflowed: grow to the reported total and classify again
    cs.stage_key.ensure((size_t)cs.h_small[6] + (cs.h_small[6] >> 2) + 1024);
    cs.stage_ty.ensure(cs.stage_key.cap);
  }
  npt = cs.h_small[3];
  nee = cs.h_small[4];
  prof_work(K_NARROW_SCAN, nov, 24.0 * g.nv + 20.0 * ((double)npt + nee));
  S.pt.ensure(4 * (size_t)npt + 4);
  S.pt_ty.ensure(npt + 1);
  S.pt_ov.ensure(npt + 1);
  S.ee.ensure(4 * (size_t)nee + 4);
  S.ee_ty.ensure(nee + 1);
  S.ee_ov.ensure(nee + 1);
  NarrowOut no{S.pt.p, S.pt_ov.p, S.ee.p, S.ee_ov.p, S.pt_ty.p, S.ee_ty.p};
  KLAUNCH(K_NARROW_WRITE, s, k_narrow_copy<<<nov, 128, 0, s>>>(nov, ovI, ovJ, cs.bin_off.p, cs.lst.p, cs.sub_cnt.p,
                                                                cs.stage_key.p, cs.stage_ty.p, cs.stage_off.p,
                                                                cs.blk_a_off.p, cs.blk_b_off.p, no));
  if (cs.h_small[7] > 0)  // some overlap was not staged: the recomputing pass writes it
    KLAUNCH(K_NARROW_WRITE, s, k_narrow_write<<<nov, NT, 0, s>>>(g, P, ds_f, ovI, ovJ, cs.bin_cnt.p, cs.bin_off.p,
                                                                  cs.lst.p, cs.vbox.p, cs.ebox.p, cs.fbox.p,
                                                                  cs.sub_cnt.p, cs.blk_a_off.p, cs.blk_b_off.p, no,
                                                                  cs.stage_off.p));
}

void cull(const Geo& g_in, const Params& P, int vtn, double alpha, CullScratch& cs, PairSet& out, double* toi_p,
          double* toi_g, cudaStream_t s) {
  Geo g = g_in;
  if (vtn != 2) g.alpha_s = nullptr;  // per-scene steps apply to trial positions only
  const bool traj = vtn == 3;
  const int nb = g.nb;
  if (!cs.h_small) {
    CK(cudaMallocHost(&cs.h_small, 64 * sizeof(int)));
    CK(cudaMallocHost(&cs.h_ll, 8 * sizeof(long long)));
  }
  // 1. projection
  if (vtn == 1) launch_project(g, 1, 0.0, s);
  else {
    launch_project(g, 2, alpha, s);
    if (traj) launch_project(g, 3, 0.0, s);
  }
  // 2-3. body boxes and overlaps
  cs.bbox.ensure(6 * (size_t)nb);
  cs.bbox_f.ensure(6 * (size_t)nb);
  cs.cnt_all.ensure(nb + 1);
  cs.cnt_up.ensure(nb + 1);
  cs.up_ptr.ensure(nb + 1);
  PairSet& S = out;
  S.row_ptr.ensure(nb + 1);
  KLAUNCH(K_BODY_BOXES, s, k_body_boxes<<<nblk(nb, 128), 128, 0, s>>>(g, vtn, alpha, cs.bbox.p, cs.bbox_f.p));
  KLAUNCH(K_OV_COUNT, s, k_ov_count<<<nblk((long long)nb * 32, 256), 256, 0, s>>>(g, cs.bbox.p, cs.bbox_f.p, cs.cnt_all.p,
                                                                                  cs.cnt_up.p));
  cs.tmp_int.ensure(64);
  int* d_tot = cs.tmp_int.p;  // [0] nnz, [1] nov, [2] list entries, [3] PT, [4] EE, [5] VG, [6] staged,
                              // [7] overlaps left to the recomputing write pass
  scan_exclusive_int(cs.cnt_all.p, S.row_ptr.p, nb, d_tot, s, cs.vflag_cnt);
  scan_exclusive_int(cs.cnt_up.p, cs.up_ptr.p, nb, d_tot + 1, s, cs.vflag_cnt);
  // the vertex-ground pairs need only the positions: counted now, read with the overlaps
  if (!traj) vg_count(g, P, cs, s);
  CK(cudaMemcpyAsync(cs.h_small, d_tot, 6 * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  int nnz = cs.h_small[0], nov = cs.h_small[1];
  const int nvg = traj ? 0 : cs.h_small[5];
  CK(cudaMemcpyAsync(S.row_ptr.p + nb, d_tot, sizeof(int), cudaMemcpyDeviceToDevice, s));
  S.nnz = nnz;
  S.nov = nov;
  S.col.ensure(nnz + 1);
  S.upidx.ensure(nnz + 1);
  cs.rowid.ensure(nnz + 1);
  S.ovI.ensure(nov + 1);
  S.ovJ.ensure(nov + 1);
  cs.ovcull.ensure(6 * (size_t)nov + 6);
  cs.ovcull_f.ensure(6 * (size_t)nov + 6);
  KLAUNCH(K_OV_FILL, s, k_ov_fill<<<nblk((long long)nb * 32, 256), 256, 0, s>>>(g, cs.bbox.p, cs.bbox_f.p, S.row_ptr.p, cs.up_ptr.p, S.col.p,
                                                          cs.rowid.p, S.upidx.p, S.ovI.p, S.ovJ.p, cs.ovcull.p,
                                                          cs.ovcull_f.p));
  if (nnz) {
    KLAUNCH(K_OV_LOWER, s, k_ov_lower<<<nblk(nnz, 256), 256, 0, s>>>(nnz, S.row_ptr.p, S.col.p, cs.rowid.p, S.upidx.p));
  }
  // 4. primitive boxes and binning
  cs.vbox.ensure(6 * (size_t)g.nv + 6);
  cs.ebox.ensure(6 * (size_t)g.ne + 6);
  cs.fbox.ensure(6 * (size_t)g.nf + 6);
  if (g.nv > 0) KLAUNCH(K_PRIM_BOXES, s, k_vert_boxes<<<nblk(g.nv, 256), 256, 0, s>>>(g, traj, cs.vbox.p));
  if (g.ne + g.nf > 0) {
    KLAUNCH(K_PRIM_BOXES, s, k_prim_boxes<<<nblk((long long)g.ne + g.nf, 256), 256, 0, s>>>(g, cs.vbox.p, cs.ebox.p,
                                                                                             cs.fbox.p));
  }
  int nlst = 0;
  if (nov > 0) {
    cs.bin_cnt.ensure(6 * (size_t)nov + 6);
    cs.bin_off.ensure(6 * (size_t)nov + 6);
    int nw = 2 * nov;
    // list capacity = the primitive counts of both bodies of every overlap; when it fits
    // (at most 2^28 entries) one binning pass writes the lists in place
    bool once = 2ll * nov * g.max_prims < (1ll << 28);
    if (once) {
      KLAUNCH(K_BIN, s, k_bin_caps<<<nblk(6ll * nov, 256), 256, 0, s>>>(g, nov, S.ovI.p, S.ovJ.p, cs.bin_cnt.p));
    } else {
      KLAUNCH(K_BIN, s, k_bin<<<nblk((long long)nw * 32, 256), 256, 0, s>>>(g, nov, BIN_COUNT, traj, S.ovI.p, S.ovJ.p,
                                                          cs.ovcull.p, cs.ovcull_f.p, cs.vbox.p, cs.ebox.p,
                                                          cs.fbox.p, cs.bin_cnt.p, nullptr, nullptr));
    }
    scan_exclusive_int(cs.bin_cnt.p, cs.bin_off.p, 6 * nov, d_tot + 2, s, cs.vflag_cnt);
    if (once) {
      // the capacities sum to at most both bodies' primitive counts per overlap
      nlst = (int)(2ll * nov * g.max_prims);
    } else {
      CK(cudaMemcpyAsync(cs.h_small + 2, d_tot + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
      CK(cudaStreamSynchronize(s));
      nlst = cs.h_small[2];
    }
    cs.lst.ensure((size_t)nlst + 1);
    KLAUNCH(K_BIN, s, k_bin<<<nblk((long long)nw * 32, 256), 256, 0, s>>>(g, nov, once ? BIN_ONCE : BIN_WRITE, traj,
                                                        S.ovI.p, S.ovJ.p, cs.ovcull.p, cs.ovcull_f.p, cs.vbox.p,
                                                        cs.ebox.p, cs.fbox.p, cs.bin_cnt.p, cs.bin_off.p, cs.lst.p));
  }
  float ds_f = float_round_up(P.d_sqrt);
  if (traj) {
    const int nk = 2 * g.ns;
    cs.toi_key.ensure(nk);
    if (cs.h_toi_cap < nk) {
      if (cs.h_toi) CK(cudaFreeHost(cs.h_toi));
      CK(cudaMallocHost(&cs.h_toi, nk * sizeof(unsigned long long)));
      cs.h_toi_cap = nk;
    }
    double o = 1.0;
    unsigned long long b;
    memcpy(&b, &o, sizeof(b));
    KLAUNCH(K_VG_TOI, s, k_fill_u64<<<nblk(nk, 256), 256, 0, s>>>(cs.toi_key.p, nk, b | 0x8000000000000000ull));
    if (nov > 0) {
      prof_work(K_NARROW_TOI, nov, 48.0 * g.nv);  // positions at q and q + dq
      // refined with the A boxes inflated by sqrt(dhat): a little looser than the TOI
      // needs (its box phase is not inflated, so the TOIs are unchanged), and the lists
      // then hold every candidate of every configuration on the trajectory, which the
      // line-search culls of this step reuse (cull_trial)
      KLAUNCH(K_NARROW_TOI, s, k_refine<true><<<nblk(3ll * nov * 32, 256), 256, 0, s>>>(g, ds_f, nov, S.ovI.p,
                                                                                         S.ovJ.p, cs.bin_cnt.p,
                                                                                         cs.bin_off.p, cs.lst.p,
                                                                                         cs.vbox.p, cs.ebox.p,
                                                                                         cs.fbox.p));
      order_overlaps(nov, cs, s, K_NARROW_TOI);
      narrow_smem_attr();
      NarrowLaunch a{g, P, ds_f, S.ovI.p, S.ovJ.p, cs.bin_cnt.p, cs.bin_off.p, cs.lst.p, cs.vbox.p, cs.ebox.p,
                     cs.fbox.p, nullptr, cs.toi_key.p, nullptr, nullptr, nullptr, nullptr, 0, cs.order.p};
      narrow_phase(2, nov, a, cs, nullptr, s);
    }
    if (P.ground && g.nv) {
      KLAUNCH(K_VG_TOI, s, k_vg_toi<<<nblk(g.nv, 256), 256, 0, s>>>(g, P, cs.toi_key.p + 1));
    }
    CK(cudaMemcpyAsync(cs.h_toi, cs.toi_key.p, nk * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    for (int sc = 0; sc < g.ns; ++sc) {
      if (toi_p) toi_p[sc] = key_to_double(cs.h_toi[2 * sc]);
      if (toi_g) toi_g[sc] = key_to_double(cs.h_toi[2 * sc + 1]);
    }
    return;
  }
  // 5. narrow phase per overlap: counts, scan, ordered write
  int npt = 0, nee = 0;
  if (nov > 0) {
    KLAUNCH(K_NARROW_SCAN, s, k_refine<true><<<nblk(3ll * nov * 32, 256), 256, 0, s>>>(g, ds_f, nov, S.ovI.p,
                                                                                       S.ovJ.p, cs.bin_cnt.p,
                                                                                       cs.bin_off.p, cs.lst.p,
                                                                                       cs.vbox.p, cs.ebox.p, cs.fbox.p));
    order_overlaps(nov, cs, s, K_NARROW_SCAN);
    narrow_pairs(g, P, ds_f, nov, S.ovI.p, S.ovJ.p, cs, S, npt, nee, s);
  }
  S.npt = npt;
  S.nee = nee;
  // 6. vertex-ground pairs (counted before the overlaps were read)
  vg_write(g, P, cs, S, nvg, s);
}

// Line-search cull at q + alpha dq over the broad phase of this step's trajectory cull H
// (its overlaps, and its lists binned with trajectory boxes and refined with the A boxes
// inflated by sqrt(dhat)): every configuration on the trajectory has its body overlaps
// among H's and its candidates among H's lists, and the lists keep primitive order, so
// the narrow phase at the trial configuration yields the pair set, in the order, that a
// full cull would (overlaps without pairs are extra, empty ones).
void cull_trial(const Geo& g_in, const Params& P, double alpha, CullScratch& cs, const PairSet& H, PairSet& out,
                cudaStream_t s) {
  Geo g = g_in;
  const int nb = g.nb, nov = H.nov, nnz = H.nnz;
  launch_project(g, 2, alpha, s);
  vg_count(g, P, cs, s);
  PairSet& S = out;
  S.row_ptr.ensure(nb + 1);
  S.col.ensure(nnz + 1);
  S.upidx.ensure(nnz + 1);
  S.ovI.ensure(nov + 1);
  S.ovJ.ensure(nov + 1);
  CK(cudaMemcpyAsync(S.row_ptr.p, H.row_ptr.p, (nb + 1) * sizeof(int), cudaMemcpyDeviceToDevice, s));
  if (nnz) {
    CK(cudaMemcpyAsync(S.col.p, H.col.p, nnz * sizeof(int), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(S.upidx.p, H.upidx.p, nnz * sizeof(int), cudaMemcpyDeviceToDevice, s));
  }
  if (nov) {
    CK(cudaMemcpyAsync(S.ovI.p, H.ovI.p, nov * sizeof(int), cudaMemcpyDeviceToDevice, s));
    CK(cudaMemcpyAsync(S.ovJ.p, H.ovJ.p, nov * sizeof(int), cudaMemcpyDeviceToDevice, s));
  }
  S.nnz = nnz;
  S.nov = nov;
  if (g.nv > 0) KLAUNCH(K_PRIM_BOXES, s, k_vert_boxes<<<nblk(g.nv, 256), 256, 0, s>>>(g, 0, cs.vbox.p));
  if (g.ne + g.nf > 0) {
    KLAUNCH(K_PRIM_BOXES, s, k_prim_boxes<<<nblk((long long)g.ne + g.nf, 256), 256, 0, s>>>(g, cs.vbox.p, cs.ebox.p,
                                                                                             cs.fbox.p));
  }
  int npt = 0, nee = 0, nvg = 0;
  if (nov > 0) {
    narrow_pairs(g, P, float_round_up(P.d_sqrt), nov, S.ovI.p, S.ovJ.p, cs, S, npt, nee, s);
    nvg = cs.h_small[5];
  } else {
    CK(cudaMemcpyAsync(cs.h_small + 5, cs.tmp_int.p + 5, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    nvg = cs.h_small[5];
  }
  S.npt = npt;
  S.nee = nee;
  vg_write(g, P, cs, S, nvg, s);
}

// Vertex-ground pairs in two halves around the host's read of their count (d_tot[5]):
// vg_count launches the per-block counts and their scan, vg_write the ordered write and
// the per-body segments.
void vg_count(const Geo& g, const Params& P, CullScratch& cs, cudaStream_t s) {
  cs.tmp_int.ensure(64);
  int* d_tot = cs.tmp_int.p;
  if (P.ground && g.nv) {
    int nbv = nblk(g.nv, 256);
    cs.vflag_off.ensure(nbv + 1);
    cs.vg_cnt.ensure(nbv + 1);
    KLAUNCH(K_VG, s, k_vg_count<<<nbv, 256, 0, s>>>(g, P, cs.vg_cnt.p));
    scan_exclusive_int(cs.vg_cnt.p, cs.vflag_off.p, nbv, d_tot + 5, s, cs.vflag_cnt);
  } else {
    CK(cudaMemsetAsync(d_tot + 5, 0, sizeof(int), s));
  }
}

void vg_write(const Geo& g, const Params& P, CullScratch& cs, PairSet& S, int nvg, cudaStream_t s) {
  const int nb = g.nb;
  S.vg_seg.ensure(nb + 2);
  if (P.ground && g.nv) {
    S.vg.ensure(2 * (size_t)nvg + 2);
    KLAUNCH(K_VG, s, k_vg_write<<<nblk(g.nv, 256), 256, 0, s>>>(g, P, cs.vflag_off.p, S.vg.p));
  } else {
    nvg = 0;
  }
  S.nvg = nvg;
  S.vg.ensure(2);
  KLAUNCH(K_VG, s, k_vg_seg<<<nblk(nb + 1, 256), 256, 0, s>>>(nb, nvg, S.vg.p, S.vg_seg.p));
}

void vg_pairs(const Geo& g, const Params& P, CullScratch& cs, PairSet& S, cudaStream_t s) {
  if (!cs.h_small) {
    CK(cudaMallocHost(&cs.h_small, 64 * sizeof(int)));
    CK(cudaMallocHost(&cs.h_ll, 8 * sizeof(long long)));
  }
  vg_count(g, P, cs, s);
  CK(cudaMemcpyAsync(cs.h_small + 5, cs.tmp_int.p + 5, sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  vg_write(g, P, cs, S, cs.h_small[5], s);
}

void launch_vg_toi(const Geo& g, const Params& P, unsigned long long* toi_key, cudaStream_t s) {
  if (!g.nv) return;
  KLAUNCH(K_VG_TOI, s, k_vg_toi<<<nblk(g.nv, 256), 256, 0, s>>>(g, P, toi_key + 1));
}

}  // namespace abd
