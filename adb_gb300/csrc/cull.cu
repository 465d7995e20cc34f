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
__global__ void k_project(Geo g, int which, double alpha) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= g.nv) return;
  int b = g.vbody[v];
  double qq[12];
  const double* q = (which == 0) ? g.q0 + 12 * b : g.q + 12 * b;
#pragma unroll
  for (int i = 0; i < 12; ++i) qq[i] = (which == 2) ? XA(q[i], XM(g.dq[12 * b + i], alpha)) : q[i];
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
__global__ void k_body_boxes(Geo g, int vtn, double alpha, double* bbox) {
  int b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= g.nb) return;
  box r{mk(g.rest_box[6 * b], g.rest_box[6 * b + 1], g.rest_box[6 * b + 2]),
        mk(g.rest_box[6 * b + 3], g.rest_box[6 * b + 4], g.rest_box[6 * b + 5])};
  double q[12], qt[12];
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
}

__device__ __forceinline__ box ldbox(const double* bb, int i) {
  return box{mk(bb[6 * i], bb[6 * i + 1], bb[6 * i + 2]), mk(bb[6 * i + 3], bb[6 * i + 4], bb[6 * i + 5])};
}

// 3. overlaps: one warp per body row i, j over its scene (j != i), in increasing j.
__global__ void k_ov_count(Geo g, const double* bbox, int* cnt_all, int* cnt_up) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= g.nb) return;
  int i = warp;
  box bi = ldbox(bbox, i);
  int ca = 0, cu = 0;
  for (int j0 = g.scene_beg[i]; j0 < g.scene_end[i]; j0 += 32) {
    int j = j0 + lane;
    bool hit = false;
    if (j < g.scene_end[i] && j != i) {
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

__global__ void k_ov_fill(Geo g, const double* bbox, const int* row_ptr, const int* up_ptr, int* col, int* rowid,
                          int* upidx, int* ovI, int* ovJ, double* ovcull, float* ovcull_f) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= g.nb) return;
  int i = warp;
  box bi = ldbox(bbox, i);
  int pa = row_ptr[i], pu = up_ptr[i];
  unsigned below = (1u << lane) - 1u;
  for (int j0 = g.scene_beg[i]; j0 < g.scene_end[i]; j0 += 32) {
    int j = j0 + lane;
    bool hit = false;
    box c;
    if (j < g.scene_end[i] && j != i) hit = intersection(bi, ldbox(bbox, j), c);
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
__global__ void k_prim_boxes(Geo g, int traj, float* vb, float* eb, float* fb) {
  int t = blockIdx.x * blockDim.x + threadIdx.x;
  int nv = g.nv;
  if (t < nv) {
    d3 p = ldX(g.X, nv, t);
    box b = traj ? box2(p, ldX(g.Xq, nv, t)) : box{p, p};
    put_fbox(vb + 6 * t, b);
    return;
  }
  t -= nv;
  if (t < g.ne) {
    int a = g.ev[2 * t], c = g.ev[2 * t + 1];
    d3 p0 = ldX(g.X, nv, a), p1 = ldX(g.X, nv, c);
    box b = traj ? box4(p0, p1, ldX(g.Xq, nv, a), ldX(g.Xq, nv, c)) : box2(p0, p1);
    put_fbox(eb + 6 * t, b);
    return;
  }
  t -= g.ne;
  if (t < g.nf) {
    int a = g.fv[3 * t], c = g.fv[3 * t + 1], d = g.fv[3 * t + 2];
    box b = box3(ldX(g.X, nv, a), ldX(g.X, nv, c), ldX(g.X, nv, d));
    if (traj) b = merge(box3(ldX(g.Xq, nv, a), ldX(g.Xq, nv, c), ldX(g.Xq, nv, d)), b);
    put_fbox(fb + 6 * t, b);
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
__global__ void k_bin(Geo g, int nov, int pass, int traj, const int* ovI, const int* ovJ, const double* ovcull,
                      const float* ovcull_f, const float* vb, const float* eb, const float* fb, int* cnt,
                      const int* off, int* lst) {
  int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (warp >= 2 * nov) return;
  int u = warp >> 1, side = warp & 1;
  int body = side ? ovJ[u] : ovI[u];
  float cf[6];
#pragma unroll
  for (int k = 0; k < 6; ++k) cf[k] = ovcull_f[6 * u + k];
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
    int c = 0, base = pass ? off[slot] : 0;
    for (int k0 = beg; k0 < end; k0 += 32) {
      int k = k0 + lane;
      bool hit = false;
      if (k < end && f_overlap(cf, fbx + 6 * k)) {
        box b = (kind == 0) ? vbox_exact(g, k, traj) : (kind == 1 ? ebox_exact(g, k, traj) : fbox_exact(g, k, traj));
        hit = overlaps(cull, b);
      }
      unsigned m = __ballot_sync(0xffffffffu, hit);
      if (pass && hit) lst[base + c + __popc(m & below)] = k - beg;
      c += __popc(m);
    }
    if (!pass && lane == 0) cnt[slot] = c;
  }
}

__global__ void k_cand_count(int nov, const int* cnt, long long* cc) {
  int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= nov) return;
  const int* c = cnt + 6 * u;
  cc[u] = (long long)c[0] * c[5] + (long long)c[3] * c[2] + (long long)c[1] * c[4];
}

struct Cand {
  int sub;       // 0: v(I) x f(J), 1: v(J) x f(I), 2: e(I) x e(J)
  int A, B;      // bodies of the first / second primitive
  int a, b;      // local primitive ids
};

__device__ __forceinline__ Cand decode(long long c, int nov, const long long* cand_off, const int* cnt, const int* off,
                                       const int* lst, const int* ovI, const int* ovJ, int& u_out) {
  int lo = 0, hi = nov;  // largest u with cand_off[u] <= c
  while (hi - lo > 1) {
    int mid = (lo + hi) >> 1;
    if (cand_off[mid] <= c) lo = mid;
    else hi = mid;
  }
  int u = lo;
  u_out = u;
  long long l = c - cand_off[u];
  const int* n = cnt + 6 * u;
  const int* o = off + 6 * u;
  long long s0 = (long long)n[0] * n[5], s1 = (long long)n[3] * n[2];
  Cand r;
  int I = ovI[u], J = ovJ[u];
  if (l < s0) {
    r.sub = 0;
    int i = (int)(l / n[5]), j = (int)(l % n[5]);
    r.A = I; r.a = lst[o[0] + i]; r.B = J; r.b = lst[o[5] + j];
  } else if (l < s0 + s1) {
    l -= s0;
    r.sub = 1;
    int i = (int)(l / n[2]), j = (int)(l % n[2]);
    r.A = J; r.a = lst[o[3] + i]; r.B = I; r.b = lst[o[2] + j];
  } else {
    l -= s0 + s1;
    r.sub = 2;
    int i = (int)(l / n[4]), j = (int)(l % n[4]);
    r.A = I; r.a = lst[o[1] + i]; r.B = J; r.b = lst[o[4] + j];
  }
  return r;
}

constexpr int NT = 256;   // narrow-phase threads per CTA
constexpr int NI = 8;     // candidates per thread
constexpr int NTILE = NT * NI;

__device__ __forceinline__ void finflate(const float* s, float ds, float* o) {
  o[0] = __fsub_rd(s[0], ds); o[1] = __fsub_rd(s[1], ds); o[2] = __fsub_rd(s[2], ds);
  o[3] = __fadd_ru(s[3], ds); o[4] = __fadd_ru(s[4], ds); o[5] = __fadd_ru(s[5], ds);
}

// Classifies one candidate. Returns 0 (no pair), 1 + type (PT) or 16 + type (EE).
__device__ __forceinline__ int classify(const Geo& g, const Params& P, float ds_f, const Cand& cd, const float* vb,
                                        const float* eb, const float* fb) {
  int nv = g.nv;
  if (cd.sub < 2) {
    int v = g.v_off[cd.A] + cd.a, f = g.f_off[cd.B] + cd.b;
    float vi[6];
    finflate(vb + 6 * v, ds_f, vi);
    if (!f_overlap(vi, fb + 6 * f)) return 0;
    d3 p = ldX(g.X, nv, v);
    box bv = inflate(box{p, p}, P.d_sqrt);
    d3 t0 = ldX(g.X, nv, g.fv[3 * f]), t1 = ldX(g.X, nv, g.fv[3 * f + 1]), t2 = ldX(g.X, nv, g.fv[3 * f + 2]);
    if (!overlaps(bv, box3(t0, t1, t2))) return 0;
    int ty = pt_type(p, t0, t1, t2);
    double d = pt_dist(p, t0, t1, t2, ty);
    return (d < P.dhat) ? 1 + ty : 0;
  } else {
    int ea = g.e_off[cd.A] + cd.a, ebi = g.e_off[cd.B] + cd.b;
    float ei[6];
    finflate(eb + 6 * ea, ds_f, ei);
    if (!f_overlap(ei, eb + 6 * ebi)) return 0;
    d3 a0 = ldX(g.X, nv, g.ev[2 * ea]), a1 = ldX(g.X, nv, g.ev[2 * ea + 1]);
    d3 b0 = ldX(g.X, nv, g.ev[2 * ebi]), b1 = ldX(g.X, nv, g.ev[2 * ebi + 1]);
    if (!overlaps(inflate(box2(a0, a1), P.d_sqrt), box2(b0, b1))) return 0;
    int ty = ee_type(a0, a1, b0, b1);
    double d = ee_dist(a0, a1, b0, b1, ty);
    return (d < P.dhat) ? 16 + ty : 0;
  }
}

// 5a. narrow phase, pass 0: flags + per-CTA counts of PT and EE pairs
__global__ void __launch_bounds__(NT) k_narrow_flags(Geo g, Params P, float ds_f, int nov, long long total,
                                                     const long long* cand_off, const int* cnt, const int* off,
                                                     const int* lst, const int* ovI, const int* ovJ, const float* vb,
                                                     const float* eb, const float* fb, uint8_t* flags, int* blk_pt,
                                                     int* blk_ee) {
  __shared__ int sp[NT / 32], se[NT / 32];
  long long base = (long long)blockIdx.x * NTILE;
  int cpt = 0, cee = 0;
#pragma unroll 1
  for (int k = 0; k < NI; ++k) {
    long long c = base + (long long)k * NT + threadIdx.x;
    int f = 0;
    if (c < total) {
      int u;
      Cand cd = decode(c, nov, cand_off, cnt, off, lst, ovI, ovJ, u);
      f = classify(g, P, ds_f, cd, vb, eb, fb);
      flags[c] = (uint8_t)f;
    }
    cpt += (f >= 1 && f < 16);
    cee += (f >= 16);
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    cpt += __shfl_xor_sync(0xffffffffu, cpt, o);
    cee += __shfl_xor_sync(0xffffffffu, cee, o);
  }
  if (lane == 0) { sp[w] = cpt; se[w] = cee; }
  __syncthreads();
  if (threadIdx.x == 0) {
    int a = 0, b = 0;
    for (int i = 0; i < NT / 32; ++i) { a += sp[i]; b += se[i]; }
    blk_pt[blockIdx.x] = a;
    blk_ee[blockIdx.x] = b;
  }
}

// 5b. narrow phase, pass 1: ordered compaction of the flagged candidates
__global__ void __launch_bounds__(NT) k_narrow_write(int nov, long long total, const long long* cand_off,
                                                     const int* cnt, const int* off, const int* lst, const int* ovI,
                                                     const int* ovJ, const uint8_t* flags, const int* blk_pt_off,
                                                     const int* blk_ee_off, int* pt, int8_t* pt_ty, int* pt_ov,
                                                     int* ee, int8_t* ee_ty, int* ee_ov) {
  __shared__ int wp[NT / 32], we[NT / 32];
  long long base = (long long)blockIdx.x * NTILE;
  int run_pt = blk_pt_off[blockIdx.x], run_ee = blk_ee_off[blockIdx.x];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  unsigned below = (1u << lane) - 1u;
#pragma unroll 1
  for (int k = 0; k < NI; ++k) {
    long long c = base + (long long)k * NT + threadIdx.x;
    int f = (c < total) ? flags[c] : 0;
    bool ip = f >= 1 && f < 16, ie = f >= 16;
    unsigned mp = __ballot_sync(0xffffffffu, ip), me = __ballot_sync(0xffffffffu, ie);
    if (lane == 0) { wp[w] = __popc(mp); we[w] = __popc(me); }
    __syncthreads();
    int pre_p = 0, pre_e = 0, tot_p = 0, tot_e = 0;
    for (int i = 0; i < NT / 32; ++i) {
      if (i < w) { pre_p += wp[i]; pre_e += we[i]; }
      tot_p += wp[i];
      tot_e += we[i];
    }
    if (ip || ie) {
      int u;
      Cand cd = decode(c, nov, cand_off, cnt, off, lst, ovI, ovJ, u);
      if (ip) {
        int idx = run_pt + pre_p + __popc(mp & below);
        pt[4 * idx] = cd.A; pt[4 * idx + 1] = cd.a; pt[4 * idx + 2] = cd.B; pt[4 * idx + 3] = cd.b;
        pt_ty[idx] = (int8_t)(f - 1);
        pt_ov[idx] = u;
      } else {
        int idx = run_ee + pre_e + __popc(me & below);
        ee[4 * idx] = cd.A; ee[4 * idx + 1] = cd.a; ee[4 * idx + 2] = cd.B; ee[4 * idx + 3] = cd.b;
        ee_ty[idx] = (int8_t)(f - 16);
        ee_ov[idx] = u;
      }
    }
    run_pt += tot_p;
    run_ee += tot_e;
    __syncthreads();
  }
}

// Order-preserving key of a double for atomicMin on unsigned 64-bit.
__device__ __forceinline__ unsigned long long dkey(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

// 5c. trajectory narrow phase: time of impact (atomic min over candidates)
__global__ void __launch_bounds__(NT) k_narrow_toi(Geo g, int nov, long long total, const long long* cand_off,
                                                   const int* cnt, const int* off, const int* lst, const int* ovI,
                                                   const int* ovJ, const float* vb, const float* eb, const float* fb,
                                                   unsigned long long* toi_key) {
  long long base = (long long)blockIdx.x * NTILE;
  double tmin = 1.0;
  int nv = g.nv;
#pragma unroll 1
  for (int k = 0; k < NI; ++k) {
    long long c = base + (long long)k * NT + threadIdx.x;
    if (c >= total) break;
    int u;
    Cand cd = decode(c, nov, cand_off, cnt, off, lst, ovI, ovJ, u);
    if (cd.sub < 2) {
      int v = g.v_off[cd.A] + cd.a, f = g.f_off[cd.B] + cd.b;
      if (!f_overlap(vb + 6 * v, fb + 6 * f)) continue;
      d3 v1 = ldX(g.X, nv, v), v0 = ldX(g.Xq, nv, v);
      int i0 = g.fv[3 * f], i1 = g.fv[3 * f + 1], i2 = g.fv[3 * f + 2];
      d3 f1[3] = {ldX(g.X, nv, i0), ldX(g.X, nv, i1), ldX(g.X, nv, i2)};
      d3 f0[3] = {ldX(g.Xq, nv, i0), ldX(g.Xq, nv, i1), ldX(g.Xq, nv, i2)};
      box bv = box2(v0, v1);
      box bf = merge(box3(f0[0], f0[1], f0[2]), box3(f1[0], f1[1], f1[2]));
      if (!overlaps(bv, bf)) continue;
      tmin = dmin(tmin, pt_collision_time(v0, f0, v1, f1));
    } else {
      int ea = g.e_off[cd.A] + cd.a, ebi = g.e_off[cd.B] + cd.b;
      if (!f_overlap(eb + 6 * ea, eb + 6 * ebi)) continue;
      int a0 = g.ev[2 * ea], a1 = g.ev[2 * ea + 1], b0 = g.ev[2 * ebi], b1 = g.ev[2 * ebi + 1];
      d3 A1[2] = {ldX(g.X, nv, a0), ldX(g.X, nv, a1)}, A0[2] = {ldX(g.Xq, nv, a0), ldX(g.Xq, nv, a1)};
      d3 B1[2] = {ldX(g.X, nv, b0), ldX(g.X, nv, b1)}, B0[2] = {ldX(g.Xq, nv, b0), ldX(g.Xq, nv, b1)};
      if (!overlaps(box4(A0[0], A0[1], A1[0], A1[1]), box4(B0[0], B0[1], B1[0], B1[1]))) continue;
      tmin = dmin(tmin, ee_collision_time(A0, B0, A1, B1));
    }
  }
  if (tmin < 1.0) atomicMin(toi_key, dkey(tmin));
}

// 6a. vertex-ground pairs: flags + per-CTA counts, then ordered write
__global__ void k_vg_count(Geo g, Params P, int* blk_cnt) {
  __shared__ int sh[32];
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  bool hit = false;
  if (v < g.nv) {
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
  if (v < g.nv) {
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

// 6b. ground time of impact (collision.cpp:83-105)
__global__ void k_vg_toi(Geo g, Params P, unsigned long long* toi_key) {
  int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= g.nv) return;
  double d2 = XA(g.X[g.nv + v], P.ground_offset);
  if (d2 < 0) {
    double d1 = XA(g.Xq[g.nv + v], P.ground_offset);
    double t = XD(d1, XS(d1, d2));
    if (t < 1.0) atomicMin(toi_key, dkey(t));
  }
}

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

// Smallest float >= d (host side).
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

void launch_project(const Geo& g, int which, double alpha, cudaStream_t s) {
  if (g.nv == 0) return;
  KLAUNCH(K_PROJECT, s, k_project<<<nblk(g.nv, 256), 256, 0, s>>>(g, which, alpha));
  prof_work(K_PROJECT, g.nv, 48.0 * g.nv);  // rest read + world write per vertex
}

void cull(const Geo& g, const Params& P, int vtn, double alpha, CullScratch& cs, PairSet& out, double* toi_p,
          double* toi_g, cudaStream_t s) {
  const bool traj = vtn == 3;
  const int nb = g.nb;
  if (!cs.h_small) {
    CK(cudaMallocHost(&cs.h_small, 64 * sizeof(int)));
    CK(cudaMallocHost(&cs.h_ll, 8 * sizeof(long long)));
    CK(cudaMallocHost(&cs.h_toi, 4 * sizeof(unsigned long long)));
  }
  // 1. projection
  if (vtn == 1) launch_project(g, 1, 0.0, s);
  else {
    launch_project(g, 2, alpha, s);
    if (traj) launch_project(g, 3, 0.0, s);
  }
  // 2-3. body boxes and overlaps
  cs.bbox.ensure(6 * (size_t)nb);
  cs.cnt_all.ensure(nb + 1);
  cs.cnt_up.ensure(nb + 1);
  cs.up_ptr.ensure(nb + 1);
  PairSet& S = out;
  S.row_ptr.ensure(nb + 1);
  KLAUNCH(K_BODY_BOXES, s, k_body_boxes<<<nblk(nb, 128), 128, 0, s>>>(g, vtn, alpha, cs.bbox.p));
  KLAUNCH(K_OV_COUNT, s, k_ov_count<<<nblk((long long)nb * 32, 256), 256, 0, s>>>(g, cs.bbox.p, cs.cnt_all.p, cs.cnt_up.p));
  cs.tmp_int.ensure(64);
  int* d_tot = cs.tmp_int.p;  // [0] nnz, [1] nov
  scan_exclusive_int(cs.cnt_all.p, S.row_ptr.p, nb, d_tot, s, cs.vflag_cnt);
  scan_exclusive_int(cs.cnt_up.p, cs.up_ptr.p, nb, d_tot + 1, s, cs.vflag_cnt);
  CK(cudaMemcpyAsync(cs.h_small, d_tot, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  int nnz = cs.h_small[0], nov = cs.h_small[1];
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
  KLAUNCH(K_OV_FILL, s, k_ov_fill<<<nblk((long long)nb * 32, 256), 256, 0, s>>>(g, cs.bbox.p, S.row_ptr.p, cs.up_ptr.p, S.col.p,
                                                          cs.rowid.p, S.upidx.p, S.ovI.p, S.ovJ.p, cs.ovcull.p,
                                                          cs.ovcull_f.p));
  if (nnz) {
    KLAUNCH(K_OV_LOWER, s, k_ov_lower<<<nblk(nnz, 256), 256, 0, s>>>(nnz, S.row_ptr.p, S.col.p, cs.rowid.p, S.upidx.p));
  }
  // 4. primitive boxes and binning
  cs.vbox.ensure(6 * (size_t)g.nv + 6);
  cs.ebox.ensure(6 * (size_t)g.ne + 6);
  cs.fbox.ensure(6 * (size_t)g.nf + 6);
  long long nprim = (long long)g.nv + g.ne + g.nf;
  KLAUNCH(K_PRIM_BOXES, s, k_prim_boxes<<<nblk(nprim, 256), 256, 0, s>>>(g, traj, cs.vbox.p, cs.ebox.p, cs.fbox.p));
  long long total = 0;
  if (nov > 0) {
    cs.bin_cnt.ensure(6 * (size_t)nov + 6);
    cs.bin_off.ensure(6 * (size_t)nov + 6);
    int nw = 2 * nov;
    KLAUNCH(K_BIN, s, k_bin<<<nblk((long long)nw * 32, 256), 256, 0, s>>>(g, nov, 0, traj, S.ovI.p, S.ovJ.p, cs.ovcull.p,
                                                        cs.ovcull_f.p, cs.vbox.p, cs.ebox.p, cs.fbox.p, cs.bin_cnt.p,
                                                        nullptr, nullptr));
    scan_exclusive_int(cs.bin_cnt.p, cs.bin_off.p, 6 * nov, d_tot + 2, s, cs.vflag_cnt);
    cs.cand_cnt.ensure(nov + 1);
    cs.cand_off.ensure(nov + 2);
    KLAUNCH(K_CAND_COUNT, s, k_cand_count<<<nblk(nov, 256), 256, 0, s>>>(nov, cs.bin_cnt.p, cs.cand_cnt.p));
    scan_exclusive_ll(cs.cand_cnt.p, cs.cand_off.p, nov, cs.cand_off.p + nov, s, cs.tmp_ll);
    CK(cudaMemcpyAsync(cs.h_small + 2, d_tot + 2, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(cs.h_ll, cs.cand_off.p + nov, sizeof(long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    int nlst = cs.h_small[2];
    total = cs.h_ll[0];
    cs.lst.ensure((size_t)nlst + 1);
    KLAUNCH(K_BIN, s, k_bin<<<nblk((long long)nw * 32, 256), 256, 0, s>>>(g, nov, 1, traj, S.ovI.p, S.ovJ.p, cs.ovcull.p,
                                                        cs.ovcull_f.p, cs.vbox.p, cs.ebox.p, cs.fbox.p, cs.bin_cnt.p,
                                                        cs.bin_off.p, cs.lst.p));
  }
  float ds_f = float_round_up(P.d_sqrt);
  int ntile = (int)((total + NTILE - 1) / NTILE);
  if (traj) {
    cs.toi_key.ensure(2);
    unsigned long long one[2];
    double o = 1.0;
    unsigned long long b;
    memcpy(&b, &o, sizeof(b));
    one[0] = one[1] = b | 0x8000000000000000ull;
    CK(cudaMemcpyAsync(cs.toi_key.p, one, sizeof(one), cudaMemcpyHostToDevice, s));
    if (total > 0) {
      prof_work(K_NARROW_TOI, (double)total, 48.0 * g.nv);  // positions at q and q + dq
      KLAUNCH(K_NARROW_TOI, s, k_narrow_toi<<<ntile, NT, 0, s>>>(g, nov, total, cs.cand_off.p, cs.bin_cnt.p, cs.bin_off.p, cs.lst.p, S.ovI.p,
                                        S.ovJ.p, cs.vbox.p, cs.ebox.p, cs.fbox.p, cs.toi_key.p));
    }
    if (P.ground && g.nv) {
      KLAUNCH(K_VG_TOI, s, k_vg_toi<<<nblk(g.nv, 256), 256, 0, s>>>(g, P, cs.toi_key.p + 1));
    }
    CK(cudaMemcpyAsync(cs.h_toi, cs.toi_key.p, 2 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    *toi_p = key_to_double(cs.h_toi[0]);
    *toi_g = key_to_double(cs.h_toi[1]);
    return;
  }
  // 5. narrow phase with ordered compaction
  int npt = 0, nee = 0;
  if (total > 0) {
    cs.flags.ensure((size_t)total + 1);
    cs.blk_a.ensure(ntile + 1);
    cs.blk_b.ensure(ntile + 1);
    cs.blk_a_off.ensure(ntile + 1);
    cs.blk_b_off.ensure(ntile + 1);
    KLAUNCH(K_NARROW_FLAGS, s, k_narrow_flags<<<ntile, NT, 0, s>>>(g, P, ds_f, nov, total, cs.cand_off.p, cs.bin_cnt.p, cs.bin_off.p, cs.lst.p,
                                        S.ovI.p, S.ovJ.p, cs.vbox.p, cs.ebox.p, cs.fbox.p, cs.flags.p, cs.blk_a.p,
                                        cs.blk_b.p));
    scan_exclusive_int(cs.blk_a.p, cs.blk_a_off.p, ntile, d_tot + 3, s, cs.vflag_cnt);
    scan_exclusive_int(cs.blk_b.p, cs.blk_b_off.p, ntile, d_tot + 4, s, cs.vflag_cnt);
    CK(cudaMemcpyAsync(cs.h_small + 3, d_tot + 3, 2 * sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    npt = cs.h_small[3];
    nee = cs.h_small[4];
    prof_work(K_NARROW_FLAGS, (double)total, 24.0 * g.nv + 20.0 * ((double)npt + nee));
    S.pt.ensure(4 * (size_t)npt + 4);
    S.pt_ty.ensure(npt + 1);
    S.pt_ov.ensure(npt + 1);
    S.ee.ensure(4 * (size_t)nee + 4);
    S.ee_ty.ensure(nee + 1);
    S.ee_ov.ensure(nee + 1);
    KLAUNCH(K_NARROW_WRITE, s, k_narrow_write<<<ntile, NT, 0, s>>>(nov, total, cs.cand_off.p, cs.bin_cnt.p, cs.bin_off.p, cs.lst.p, S.ovI.p,
                                        S.ovJ.p, cs.flags.p, cs.blk_a_off.p, cs.blk_b_off.p, S.pt.p, S.pt_ty.p,
                                        S.pt_ov.p, S.ee.p, S.ee_ty.p, S.ee_ov.p));
  }
  S.npt = npt;
  S.nee = nee;
  // 6. vertex-ground pairs
  int nvg = 0;
  S.vg_seg.ensure(nb + 2);
  if (P.ground && g.nv) {
    int nbv = nblk(g.nv, 256);
    cs.vflag_off.ensure(nbv + 1);
    cs.blk_a.ensure(nbv + 1);
    KLAUNCH(K_VG, s, k_vg_count<<<nbv, 256, 0, s>>>(g, P, cs.blk_a.p));
    scan_exclusive_int(cs.blk_a.p, cs.vflag_off.p, nbv, d_tot + 5, s, cs.vflag_cnt);
    CK(cudaMemcpyAsync(cs.h_small + 5, d_tot + 5, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    nvg = cs.h_small[5];
    S.vg.ensure(2 * (size_t)nvg + 2);
    KLAUNCH(K_VG, s, k_vg_write<<<nbv, 256, 0, s>>>(g, P, cs.vflag_off.p, S.vg.p));
  }
  S.nvg = nvg;
  KLAUNCH(K_VG, s, k_vg_seg<<<nblk(nb + 1, 256), 256, 0, s>>>(nb, nvg, S.vg.p, S.vg_seg.p));
}

}  // namespace abd
