// Spatial-hash broad phase (the reference's iaabb-even path): gen_collision_set
// (model/col_set.cpp:20-339, global point / edge / triangle lists) and
// step_size_upper_bound (model/upper_bound.cpp:16-277) over the hash grid of
// model/spatial_hashing.cpp:11-211.
//
// Grid: a point x lies in cell int(max(x - min_xyz, 0) / dx) per axis; a cell's bucket
// keeps the low xyz_bits bits of each coordinate (spatial_hashing.cpp:11-21), so cells
// that agree modulo 2^xyz_bits share a bucket. Registration writes one 64-bit key
// (bucket << 32 | primitive) per covered cell; the keys are sorted, so every bucket is a
// contiguous, ordered run. A query walks the buckets of its cell range in the
// reference's loop order; a registered primitive is taken in the first query cell whose
// bucket holds it (the reference gathers, sorts and de-duplicates per query).
//
// Distance culling keeps the pairs of different bodies with squared distance below
// dhat * safe_factor^2 (PT: vertex of any body against a triangle; EE: edges of bodies
// I < J) and orders them as the overlap-based path does (body pair, then vertex-on-I,
// vertex-on-J, edge-edge, each by primitive ids), building the body-pair CSR the
// assembly walks. The reference appends its threads' pairs in scheduling order, so only
// the set is defined there. The trajectory bound takes the exact time of impact of every
// candidate that shares a bucket (edge trajectories registered by their start position
// unless the fix flag is set, as upper_bound.cpp:151 does), or the d_sqrt / |dq|_1
// bound lowered by the current pairs' times of impact.
#include <algorithm>
#include <cstring>
#include <stdexcept>

#include "abd_engine.h"
#include "abd_exact.cuh"

namespace abd {

namespace {

inline int nblk(long long n, int t) { return (int)((n + t - 1) / t); }

// Order-preserving key of a double for atomicMin on unsigned 64-bit.
__device__ __forceinline__ unsigned long long dkey(double x) {
  unsigned long long b = (unsigned long long)__double_as_longlong(x);
  return (b >> 63) ? ~b : (b | 0x8000000000000000ull);
}

__device__ __forceinline__ d3 ldX(const double* X, int nv, int v) { return mk(X[v], X[nv + v], X[2 * nv + v]); }

struct ShGrid {
  double mn, dx;
  int bits;
};

__device__ __forceinline__ int sh_cell(double x, const ShGrid& G) {
  double t = XS(x, G.mn);
  t = t < 0.0 ? 0.0 : t;
  return (int)XD(t, G.dx);
}
__device__ __forceinline__ void sh_cells(const d3& p, const ShGrid& G, int* c) {
  c[0] = sh_cell(p.x, G);
  c[1] = sh_cell(p.y, G);
  c[2] = sh_cell(p.z, G);
}
__device__ __forceinline__ unsigned sh_hash(int i, int j, int k, int bits) {
  unsigned m = (1u << bits) - 1u;
  return ((((unsigned)i & m) << bits | ((unsigned)j & m)) << bits) | ((unsigned)k & m);
}
__device__ __forceinline__ d3 dmin3(const d3& a, const d3& b) { return mk(dmin(a.x, b.x), dmin(a.y, b.y), dmin(a.z, b.z)); }
__device__ __forceinline__ d3 dmax3(const d3& a, const d3& b) { return mk(dmax(a.x, b.x), dmax(a.y, b.y), dmax(a.z, b.z)); }

// First cell coordinate a >= l whose bucket residue lies in the residues of [rl, ru].
__device__ __forceinline__ int first_hit(int l, int rl, int ru, int bits) {
  const int M = 1 << bits, m = M - 1;
  int L = ru - rl + 1;
  if (L >= M) return l;
  int off = ((l & m) - (rl & m)) & m;
  return off < L ? l : l + (M - off);
}

// Registered box of a primitive. kind 0: vertex (point, or q -> target segment when
// traj); kind 1: edge (segment at the target, or at q when traj, widened to the target
// positions when fix_edge).
__device__ __forceinline__ void reg_box(const Geo& g, int kind, int id, int traj, int fix_edge, d3& lo, d3& hi) {
  if (kind == 0) {
    d3 p = ldX(g.X, g.nv, id);
    if (traj) {
      d3 p0 = ldX(g.Xq, g.nv, id);
      lo = dmin3(p0, p);
      hi = dmax3(p0, p);
    } else {
      lo = hi = p;
    }
    return;
  }
  int a = g.ev[2 * id], b = g.ev[2 * id + 1];
  const double* P = traj ? g.Xq : g.X;
  d3 a0 = ldX(P, g.nv, a), a1 = ldX(P, g.nv, b);
  lo = dmin3(a0, a1);
  hi = dmax3(a0, a1);
  if (traj && fix_edge) {
    d3 b0 = ldX(g.X, g.nv, a), b1 = ldX(g.X, g.nv, b);
    lo = dmin3(lo, dmin3(b0, b1));
    hi = dmax3(hi, dmax3(b0, b1));
  }
}

__global__ void k_reg_count(Geo g, ShGrid G, int kind, int n, int traj, int fix_edge, long long* cnt) {
  int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= n) return;
  d3 lo, hi;
  reg_box(g, kind, id, traj, fix_edge, lo, hi);
  int l[3], u[3];
  sh_cells(lo, G, l);
  sh_cells(hi, G, u);
  cnt[id] = (long long)(u[0] - l[0] + 1) * (u[1] - l[1] + 1) * (u[2] - l[2] + 1);
}

__global__ void k_reg_fill(Geo g, ShGrid G, int kind, int n, int traj, int fix_edge, const long long* off,
                           unsigned long long* keys) {
  int id = blockIdx.x * blockDim.x + threadIdx.x;
  if (id >= n) return;
  d3 lo, hi;
  reg_box(g, kind, id, traj, fix_edge, lo, hi);
  int l[3], u[3];
  sh_cells(lo, G, l);
  sh_cells(hi, G, u);
  long long o = off[id];
  for (int i = l[0]; i <= u[0]; ++i)
    for (int j = l[1]; j <= u[1]; ++j)
      for (int k = l[2]; k <= u[2]; ++k)
        keys[o++] = ((unsigned long long)sh_hash(i, j, k, G.bits) << 32) | (unsigned)id;
}

__global__ void k_bucket_bounds(const unsigned long long* keys, long long n, int* bstart, int* bend) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  unsigned b = (unsigned)(keys[i] >> 32);
  if (i == 0 || (unsigned)(keys[i - 1] >> 32) != b) bstart[b] = (int)i;
  if (i == n - 1 || (unsigned)(keys[i + 1] >> 32) != b) bend[b] = (int)(i + 1);
}

struct ShQuery {
  ShGrid G;
  const unsigned long long* keys;
  const int *bstart, *bend;
  double qd;     // query box growth (d_sqrt * safe_factor); 0 for trajectories
  double thr;    // squared-distance threshold (dhat * safe_factor^2)
  double marg;   // prefilter margin: boxes farther apart than qd + marg cannot pass thr
  int traj, fix_edge;
};

__device__ __forceinline__ bool box_apart(const d3& alo, const d3& ahi, const d3& blo, const d3& bhi, double m) {
  return ahi.x < blo.x - m || blo.x > ahi.x + m || ahi.y < blo.y - m || blo.y > ahi.y + m || ahi.z < blo.z - m ||
         blo.z > ahi.z + m;
}

__device__ __forceinline__ unsigned long long pair_key(int A, int a, int B, int b, int sub) {
  unsigned long long lo = A < B ? A : B, hi = A < B ? B : A;
  return (lo << 47) | (hi << 32) | ((unsigned long long)sub << 30) | ((unsigned long long)a << 15) |
         (unsigned long long)b;
}

// PT query, thread per triangle. MODE 0: count, 1: write keys, 2: time of impact.
template <int MODE>
__global__ void k_pt_query(Geo g, ShQuery Q, const int* off, unsigned long long* out,
                           unsigned long long* toi_key, int* cnt) {
  int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= g.nf) return;
  int i0 = g.fv[3 * f], i1 = g.fv[3 * f + 1], i2 = g.fv[3 * f + 2];
  int J = g.vbody[i0];
  if (!scene_on(g, J)) {
    if (MODE == 0) cnt[f] = 0;
    return;
  }
  d3 t0 = ldX(g.X, g.nv, i0), t1 = ldX(g.X, g.nv, i1), t2 = ldX(g.X, g.nv, i2);
  d3 lo = dmin3(dmin3(t0, t1), t2), hi = dmax3(dmax3(t0, t1), t2);
  d3 f0[3], f1[3] = {t0, t1, t2};
  if (MODE == 2) {
    f0[0] = ldX(g.Xq, g.nv, i0);
    f0[1] = ldX(g.Xq, g.nv, i1);
    f0[2] = ldX(g.Xq, g.nv, i2);
    lo = dmin3(lo, dmin3(dmin3(f0[0], f0[1]), f0[2]));
    hi = dmax3(hi, dmax3(dmax3(f0[0], f0[1]), f0[2]));
  } else {
    lo = mk(XA(lo.x, -Q.qd), XA(lo.y, -Q.qd), XA(lo.z, -Q.qd));
    hi = mk(XA(hi.x, Q.qd), XA(hi.y, Q.qd), XA(hi.z, Q.qd));
  }
  int l[3], u[3];
  sh_cells(lo, Q.G, l);
  sh_cells(hi, Q.G, u);
  int c = 0;
  long long w = MODE == 1 ? off[f] : 0;
  double tmin = 1.0;
  const int f_loc = f - g.f_off[J];
  for (int i = l[0]; i <= u[0]; ++i)
    for (int j = l[1]; j <= u[1]; ++j)
      for (int k = l[2]; k <= u[2]; ++k) {
        unsigned b = sh_hash(i, j, k, Q.G.bits);
        for (int e = Q.bstart[b]; e < Q.bend[b]; ++e) {
          if (e > Q.bstart[b] && Q.keys[e] == Q.keys[e - 1]) continue;  // registered twice in one bucket
          int v = (int)(Q.keys[e] & 0xffffffffull);
          int I = g.vbody[v];
          if (I == J || g.bscene[I] != g.bscene[J]) continue;
          d3 rlo, rhi;
          reg_box(g, 0, v, Q.traj, 0, rlo, rhi);
          int rl[3], ru[3];
          sh_cells(rlo, Q.G, rl);
          sh_cells(rhi, Q.G, ru);
          if (i != first_hit(l[0], rl[0], ru[0], Q.G.bits) || j != first_hit(l[1], rl[1], ru[1], Q.G.bits) ||
              k != first_hit(l[2], rl[2], ru[2], Q.G.bits))
            continue;
          if (MODE == 2) {
            tmin = dmin(tmin, pt_collision_time(ldX(g.Xq, g.nv, v), f0, ldX(g.X, g.nv, v), f1));
            continue;
          }
          d3 p = rlo;
          if (box_apart(p, p, lo, hi, Q.marg)) continue;
          int ty = pt_type(p, t0, t1, t2);
          if (!(pt_dist(p, t0, t1, t2, ty) < Q.thr)) continue;
          if (MODE == 1) out[w++] = pair_key(I, v - g.v_off[I], J, f_loc, I < J ? 0 : 1);
          ++c;
        }
      }
  if (MODE == 0) cnt[f] = c;
  if (MODE == 2 && tmin < 1.0) atomicMin(toi_key + 2 * g.bscene[J], dkey(tmin));
}

// EE query, thread per edge of body J against edges of bodies I < J.
template <int MODE>
__global__ void k_ee_query(Geo g, ShQuery Q, const int* off, unsigned long long* out,
                           unsigned long long* toi_key, int* cnt) {
  int ej = blockIdx.x * blockDim.x + threadIdx.x;
  if (ej >= g.ne) return;
  int jb0 = g.ev[2 * ej], jb1 = g.ev[2 * ej + 1];
  int J = g.vbody[jb0];
  if (!scene_on(g, J)) {
    if (MODE == 0) cnt[ej] = 0;
    return;
  }
  d3 b0 = ldX(g.X, g.nv, jb0), b1 = ldX(g.X, g.nv, jb1);
  d3 lo = dmin3(b0, b1), hi = dmax3(b0, b1);
  d3 q0[2], q1[2] = {b0, b1};
  if (MODE == 2) {
    q0[0] = ldX(g.Xq, g.nv, jb0);
    q0[1] = ldX(g.Xq, g.nv, jb1);
    lo = dmin3(lo, dmin3(q0[0], q0[1]));
    hi = dmax3(hi, dmax3(q0[0], q0[1]));
  } else {
    lo = mk(XA(lo.x, -Q.qd), XA(lo.y, -Q.qd), XA(lo.z, -Q.qd));
    hi = mk(XA(hi.x, Q.qd), XA(hi.y, Q.qd), XA(hi.z, Q.qd));
  }
  int l[3], u[3];
  sh_cells(lo, Q.G, l);
  sh_cells(hi, Q.G, u);
  int c = 0;
  long long w = MODE == 1 ? off[ej] : 0;
  double tmin = 1.0;
  const int ej_loc = ej - g.e_off[J];
  for (int i = l[0]; i <= u[0]; ++i)
    for (int j = l[1]; j <= u[1]; ++j)
      for (int k = l[2]; k <= u[2]; ++k) {
        unsigned b = sh_hash(i, j, k, Q.G.bits);
        for (int e = Q.bstart[b]; e < Q.bend[b]; ++e) {
          if (e > Q.bstart[b] && Q.keys[e] == Q.keys[e - 1]) continue;  // registered twice in one bucket
          int ei = (int)(Q.keys[e] & 0xffffffffull);
          int ia0 = g.ev[2 * ei], ia1 = g.ev[2 * ei + 1];
          int I = g.vbody[ia0];
          if (I >= J || g.bscene[I] != g.bscene[J]) continue;
          d3 rlo, rhi;
          reg_box(g, 1, ei, Q.traj, Q.fix_edge, rlo, rhi);
          int rl[3], ru[3];
          sh_cells(rlo, Q.G, rl);
          sh_cells(rhi, Q.G, ru);
          if (i != first_hit(l[0], rl[0], ru[0], Q.G.bits) || j != first_hit(l[1], rl[1], ru[1], Q.G.bits) ||
              k != first_hit(l[2], rl[2], ru[2], Q.G.bits))
            continue;
          if (MODE == 2) {
            d3 a0[2] = {ldX(g.Xq, g.nv, ia0), ldX(g.Xq, g.nv, ia1)}, a1[2] = {ldX(g.X, g.nv, ia0), ldX(g.X, g.nv, ia1)};
            tmin = dmin(tmin, ee_collision_time(a0, q0, a1, q1));
            continue;
          }
          if (box_apart(rlo, rhi, lo, hi, Q.marg)) continue;
          d3 a0 = ldX(g.X, g.nv, ia0), a1 = ldX(g.X, g.nv, ia1);
          int ty = ee_type(a0, a1, b0, b1);
          if (!(ee_dist(a0, a1, b0, b1, ty) < Q.thr)) continue;
          if (MODE == 1) out[w++] = pair_key(I, ei - g.e_off[I], J, ej_loc, 2);
          ++c;
        }
      }
  if (MODE == 0) cnt[ej] = c;
  if (MODE == 2 && tmin < 1.0) atomicMin(toi_key + 2 * g.bscene[J], dkey(tmin));
}

// Sorted pair keys -> tuples, distance types (recomputed, as in the query) and the
// body-pair key of each pair.
__global__ void k_decode_pt(Geo g, int n, const unsigned long long* keys, int* pt, int8_t* ty, unsigned* bp) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  unsigned long long k = keys[p];
  int lo = (int)(k >> 47), hi = (int)((k >> 32) & 0x7fff), sub = (int)((k >> 30) & 3);
  int a = (int)((k >> 15) & 0x7fff), b = (int)(k & 0x7fff);
  int A = sub == 0 ? lo : hi, B = sub == 0 ? hi : lo;
  pt[4 * p] = A; pt[4 * p + 1] = a; pt[4 * p + 2] = B; pt[4 * p + 3] = b;
  int f = g.f_off[B] + b;
  d3 x = ldX(g.X, g.nv, g.v_off[A] + a);
  d3 t0 = ldX(g.X, g.nv, g.fv[3 * f]), t1 = ldX(g.X, g.nv, g.fv[3 * f + 1]), t2 = ldX(g.X, g.nv, g.fv[3 * f + 2]);
  ty[p] = (int8_t)pt_type(x, t0, t1, t2);
  bp[p] = (unsigned)(k >> 32);
}
__global__ void k_decode_ee(Geo g, int n, const unsigned long long* keys, int* ee, int8_t* ty, unsigned* bp) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  unsigned long long k = keys[p];
  int A = (int)(k >> 47), B = (int)((k >> 32) & 0x7fff);
  int a = (int)((k >> 15) & 0x7fff), b = (int)(k & 0x7fff);
  ee[4 * p] = A; ee[4 * p + 1] = a; ee[4 * p + 2] = B; ee[4 * p + 3] = b;
  int ea = g.e_off[A] + a, eb = g.e_off[B] + b;
  d3 a0 = ldX(g.X, g.nv, g.ev[2 * ea]), a1 = ldX(g.X, g.nv, g.ev[2 * ea + 1]);
  d3 b0 = ldX(g.X, g.nv, g.ev[2 * eb]), b1 = ldX(g.X, g.nv, g.ev[2 * eb + 1]);
  ty[p] = (int8_t)ee_type(a0, a1, b0, b1);
  bp[p] = (unsigned)(k >> 32);
}

// Body-pair keys (I << 15 | J) of both lists as 64-bit sort keys.
__global__ void k_bp_keys(int npt, const unsigned* bpt, int nee, const unsigned* bee, unsigned long long* out) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < npt) out[i] = bpt[i];
  else if (i < npt + nee) out[i] = bee[i - npt];
}
__global__ void k_unique_flags(long long n, const unsigned long long* k, int* flag) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flag[i] = (i == 0 || k[i] != k[i - 1]) ? 1 : 0;
}
__global__ void k_unique_write(long long n, const unsigned long long* k, const int* flag, const int* pos, int* ovI,
                               int* ovJ, unsigned long long* tkeys) {
  long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n || !flag[i]) return;
  int u = pos[i];
  int I = (int)(k[i] >> 15), J = (int)(k[i] & 0x7fff);
  ovI[u] = I;
  ovJ[u] = J;
  tkeys[u] = ((unsigned long long)J << 32) | (unsigned)u;  // transposed: row J, lower entry
}

__device__ __forceinline__ int lb_ov(const int* ovI, int nov, int r) {
  int lo = 0, hi = nov;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (ovI[mid] < r) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}
__device__ __forceinline__ int lb_t(const unsigned long long* t, int nov, int r) {
  int lo = 0, hi = nov;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if ((int)(t[mid] >> 32) < r) lo = mid + 1;
    else hi = mid;
  }
  return lo;
}

// Row r of the symmetric CSR: lower entries (overlaps (I, r), I ascending) then upper
// entries (overlaps (r, J), J ascending); upidx is the overlap of each entry.
__global__ void k_csr_count(int nb, int nov, const int* ovI, const unsigned long long* tkeys, int* cnt) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nb) return;
  cnt[r] = (lb_t(tkeys, nov, r + 1) - lb_t(tkeys, nov, r)) + (lb_ov(ovI, nov, r + 1) - lb_ov(ovI, nov, r));
}
__global__ void k_csr_fill(int nb, int nov, const int* ovI, const int* ovJ, const unsigned long long* tkeys,
                           const int* row_ptr, int* col, int* upidx) {
  int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= nb) return;
  int e = row_ptr[r];
  for (int t = lb_t(tkeys, nov, r), t1 = lb_t(tkeys, nov, r + 1); t < t1; ++t) {
    int u = (int)(tkeys[t] & 0xffffffffull);
    col[e] = ovI[u];
    upidx[e++] = u;
  }
  for (int u = lb_ov(ovI, nov, r), u1 = lb_ov(ovI, nov, r + 1); u < u1; ++u) {
    col[e] = ovJ[u];
    upidx[e++] = u;
  }
}

// Overlap of every pair (binary search of its body-pair key in the unique list).
__global__ void k_pair_ov(int n, const unsigned* bp, int nov, const int* ovI, const int* ovJ, int* pov) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  unsigned key = bp[p];
  int lo = 0, hi = nov;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    unsigned km = ((unsigned)ovI[mid] << 15) | (unsigned)ovJ[mid];
    if (km < key) lo = mid + 1;
    else hi = mid;
  }
  pov[p] = lo;
}

// step_size_upper_bound without full_ccd: per scene, d_sqrt / 2 / max_I |dq_I|_1 * sf,
// capped at 1 (upper_bound.cpp:232-233).
__global__ void __launch_bounds__(256) k_norm1_bound(const int* sc_beg, const int* sc_end, const double* dq,
                                                    double half_ds, double sf, unsigned long long* toi_key) {
  __shared__ double sh[8];
  int s = blockIdx.x;
  double m = 0.0;
  for (int b = sc_beg[s] + (int)threadIdx.x; b < sc_end[s]; b += blockDim.x) {
    double a = 0.0;
    for (int i = 0; i < 12; ++i) a += fabs(dq[12 * b + i]);
    m = dmax(m, a);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = dmax(m, __shfl_xor_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = dmax(m, sh[w]);
    double t = XM(XD(half_ds, m), sf);
    t = t < 1.0 ? t : 1.0;
    atomicMin(toi_key + 2 * s, dkey(t));
  }
}

// ... lowered by the times of impact of the current pairs.
__global__ void k_pair_toi(Geo g, int npt, const int* pt, int nee, const int* ee, unsigned long long* toi_key) {
  int p = blockIdx.x * blockDim.x + threadIdx.x;
  double t = 1.0;
  int A;
  if (p < npt) {
    A = pt[4 * p];
    int v = g.v_off[A] + pt[4 * p + 1], B = pt[4 * p + 2], f = g.f_off[B] + pt[4 * p + 3];
    int i0 = g.fv[3 * f], i1 = g.fv[3 * f + 1], i2 = g.fv[3 * f + 2];
    d3 f0[3] = {ldX(g.Xq, g.nv, i0), ldX(g.Xq, g.nv, i1), ldX(g.Xq, g.nv, i2)};
    d3 f1[3] = {ldX(g.X, g.nv, i0), ldX(g.X, g.nv, i1), ldX(g.X, g.nv, i2)};
    t = pt_collision_time(ldX(g.Xq, g.nv, v), f0, ldX(g.X, g.nv, v), f1);
  } else if (p < npt + nee) {
    int q = p - npt;
    A = ee[4 * q];
    int ea = g.e_off[A] + ee[4 * q + 1], B = ee[4 * q + 2], eb = g.e_off[B] + ee[4 * q + 3];
    d3 a0[2] = {ldX(g.Xq, g.nv, g.ev[2 * ea]), ldX(g.Xq, g.nv, g.ev[2 * ea + 1])};
    d3 a1[2] = {ldX(g.X, g.nv, g.ev[2 * ea]), ldX(g.X, g.nv, g.ev[2 * ea + 1])};
    d3 b0[2] = {ldX(g.Xq, g.nv, g.ev[2 * eb]), ldX(g.Xq, g.nv, g.ev[2 * eb + 1])};
    d3 b1[2] = {ldX(g.X, g.nv, g.ev[2 * eb]), ldX(g.X, g.nv, g.ev[2 * eb + 1])};
    t = ee_collision_time(a0, b0, a1, b1);
  } else {
    return;
  }
  if (t < 1.0) atomicMin(toi_key + 2 * g.bscene[A], dkey(t));
}
__global__ void k_vg_pair_toi(Geo g, Params P, int nvg, const int* vg, unsigned long long* toi_key) {
  int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nvg) return;
  int b = vg[2 * k], v = g.v_off[b] + vg[2 * k + 1];
  double d2 = XA(g.X[g.nv + v], P.ground_offset);
  if (!(d2 < 0)) return;
  double d1 = XA(g.Xq[g.nv + v], P.ground_offset);
  double t = XD(d1, XS(d1, d2));
  if (t < 1.0) atomicMin(toi_key + 2 * g.bscene[b], dkey(t));
}

__global__ void k_fill_key(unsigned long long* p, int n, unsigned long long v) {
  int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = v;
}

double key_to_double_h(unsigned long long k) {
  unsigned long long b = (k >> 63) ? (k & 0x7fffffffffffffffull) : ~k;
  double d;
  memcpy(&d, &b, sizeof(d));
  return d;
}

ShGrid grid_of(const ShParams& H) { return ShGrid{H.min_xyz, H.dx, H.bits}; }

}  // namespace

// Registers `n` primitives of `kind` and builds the bucket table in `T`.
static void sh_register(const Geo& g, const ShParams& H, int kind, int n, int traj, ShTable& T, cudaStream_t s) {
  ShGrid G = grid_of(H);
  T.cnt.ensure((size_t)n + 1);
  T.off.ensure((size_t)n + 1);
  size_t nbuckets = (size_t)1 << (3 * H.bits);
  T.bstart.ensure(nbuckets);
  T.bend.ensure(nbuckets);
  CK(cudaMemsetAsync(T.bstart.p, 0, nbuckets * sizeof(int), s));
  CK(cudaMemsetAsync(T.bend.p, 0, nbuckets * sizeof(int), s));
  T.n = 0;
  if (n == 0) return;
  KLAUNCH(K_SH, s, k_reg_count<<<nblk(n, 256), 256, 0, s>>>(g, G, kind, n, traj, H.fix_edge, T.cnt.p));
  scan_exclusive_ll(T.cnt.p, T.off.p, n, T.off.p + n, s, T.scan_tmp);
  long long tot = 0;
  CK(cudaMemcpyAsync(&T.h_tot, T.off.p + n, sizeof(long long), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  tot = T.h_tot;
  if (tot > (1ll << 31) - 1) throw std::invalid_argument("spatial hash: too many cell registrations (dx too small)");
  size_t cap = sort_padded_size((size_t)tot);
  T.keys.ensure(cap);
  KLAUNCH(K_SH, s, k_reg_fill<<<nblk(n, 256), 256, 0, s>>>(g, G, kind, n, traj, H.fix_edge, T.off.p, T.keys.p));
  sort_u64(T.keys.p, (size_t)tot, cap, s);
  KLAUNCH(K_SH, s, k_bucket_bounds<<<nblk(tot, 256), 256, 0, s>>>(T.keys.p, tot, T.bstart.p, T.bend.p));
  T.n = tot;
}

void sh_cull(const Geo& g, const Params& P, const ShParams& H, int vtn, double alpha, ShScratch& W, CullScratch& cs,
             PairSet& S, cudaStream_t s) {
  const int nb = g.nb;
  launch_project(g, vtn == 1 ? 1 : 2, alpha, s);
  const double sf = H.safe_factor;
  ShQuery Q;
  Q.G = grid_of(H);
  Q.qd = P.d_sqrt * sf;
  Q.thr = P.dhat * (sf * sf);
  Q.marg = 1e-6 * Q.qd;
  Q.traj = 0;
  Q.fix_edge = 0;
  if (!W.h_int) CK(cudaMallocHost(&W.h_int, 8 * sizeof(int)));
  int npt = 0, nee = 0;
  // PT: vertices registered, triangles query
  if (P.pt && g.nv && g.nf) {
    sh_register(g, H, 0, g.nv, 0, W.tab, s);
    Q.keys = W.tab.keys.p;
    Q.bstart = W.tab.bstart.p;
    Q.bend = W.tab.bend.p;
    W.qcnt.ensure((size_t)g.nf + 1);
    W.qoff.ensure((size_t)g.nf + 1);
    KLAUNCH(K_SH, s, k_pt_query<0><<<nblk(g.nf, 128), 128, 0, s>>>(g, Q, nullptr, nullptr, nullptr, W.qcnt.p));
    scan_exclusive_int(W.qcnt.p, W.qoff.p, g.nf, W.qoff.p + g.nf, s, W.scan_i);
    CK(cudaMemcpyAsync(W.h_int, W.qoff.p + g.nf, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    npt = W.h_int[0];
    W.pt_keys.ensure(sort_padded_size(npt));
    if (npt) {
      KLAUNCH(K_SH, s, k_pt_query<1><<<nblk(g.nf, 128), 128, 0, s>>>(g, Q, W.qoff.p, W.pt_keys.p, nullptr, nullptr));
      sort_u64(W.pt_keys.p, npt, W.pt_keys.cap, s);
    }
  }
  // EE: edges registered, edges of the higher body query
  if (P.ee && g.ne) {
    sh_register(g, H, 1, g.ne, 0, W.tab, s);
    Q.keys = W.tab.keys.p;
    Q.bstart = W.tab.bstart.p;
    Q.bend = W.tab.bend.p;
    W.qcnt.ensure((size_t)g.ne + 1);
    W.qoff.ensure((size_t)g.ne + 1);
    KLAUNCH(K_SH, s, k_ee_query<0><<<nblk(g.ne, 128), 128, 0, s>>>(g, Q, nullptr, nullptr, nullptr, W.qcnt.p));
    scan_exclusive_int(W.qcnt.p, W.qoff.p, g.ne, W.qoff.p + g.ne, s, W.scan_i);
    CK(cudaMemcpyAsync(W.h_int, W.qoff.p + g.ne, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    nee = W.h_int[0];
    W.ee_keys.ensure(sort_padded_size(nee));
    if (nee) {
      KLAUNCH(K_SH, s, k_ee_query<1><<<nblk(g.ne, 128), 128, 0, s>>>(g, Q, W.qoff.p, W.ee_keys.p, nullptr, nullptr));
      sort_u64(W.ee_keys.p, nee, W.ee_keys.cap, s);
    }
  }
  // tuples, types and body-pair keys
  S.npt = npt;
  S.nee = nee;
  S.pt.ensure(4 * (size_t)npt + 4);
  S.pt_ty.ensure((size_t)npt + 1);
  S.pt_ov.ensure((size_t)npt + 1);
  S.ee.ensure(4 * (size_t)nee + 4);
  S.ee_ty.ensure((size_t)nee + 1);
  S.ee_ov.ensure((size_t)nee + 1);
  W.bp_pt.ensure((size_t)npt + 1);
  W.bp_ee.ensure((size_t)nee + 1);
  if (npt) KLAUNCH(K_SH, s, k_decode_pt<<<nblk(npt, 256), 256, 0, s>>>(g, npt, W.pt_keys.p, S.pt.p, S.pt_ty.p, W.bp_pt.p));
  if (nee) KLAUNCH(K_SH, s, k_decode_ee<<<nblk(nee, 256), 256, 0, s>>>(g, nee, W.ee_keys.p, S.ee.p, S.ee_ty.p, W.bp_ee.p));
  // unique body pairs -> overlaps and the symmetric CSR
  long long nbp = (long long)npt + nee;
  int nov = 0;
  W.bp_all.ensure(sort_padded_size(nbp));
  W.flag.ensure((size_t)nbp + 1);
  W.pos.ensure((size_t)nbp + 1);
  if (nbp) {
    KLAUNCH(K_SH, s, k_bp_keys<<<nblk(nbp, 256), 256, 0, s>>>(npt, W.bp_pt.p, nee, W.bp_ee.p, W.bp_all.p));
    sort_u64(W.bp_all.p, nbp, W.bp_all.cap, s);
    KLAUNCH(K_SH, s, k_unique_flags<<<nblk(nbp, 256), 256, 0, s>>>(nbp, W.bp_all.p, W.flag.p));
    scan_exclusive_int(W.flag.p, W.pos.p, (int)nbp, W.pos.p + nbp, s, W.scan_i);
    CK(cudaMemcpyAsync(W.h_int, W.pos.p + nbp, sizeof(int), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    nov = W.h_int[0];
  }
  S.nov = nov;
  S.ovI.ensure(nov + 1);
  S.ovJ.ensure(nov + 1);
  W.tkeys.ensure(sort_padded_size(nov));
  if (nov) {
    KLAUNCH(K_SH, s, k_unique_write<<<nblk(nbp, 256), 256, 0, s>>>(nbp, W.bp_all.p, W.flag.p, W.pos.p, S.ovI.p, S.ovJ.p,
                                                                  W.tkeys.p));
    sort_u64(W.tkeys.p, nov, W.tkeys.cap, s);
  }
  S.row_ptr.ensure(nb + 1);
  cs.cnt_all.ensure(nb + 1);
  KLAUNCH(K_SH, s, k_csr_count<<<nblk(nb, 256), 256, 0, s>>>(nb, nov, S.ovI.p, W.tkeys.p, cs.cnt_all.p));
  scan_exclusive_int(cs.cnt_all.p, S.row_ptr.p, nb, S.row_ptr.p + nb, s, W.scan_i);
  S.nnz = 2 * nov;
  S.col.ensure(S.nnz + 1);
  S.upidx.ensure(S.nnz + 1);
  KLAUNCH(K_SH, s, k_csr_fill<<<nblk(nb, 256), 256, 0, s>>>(nb, nov, S.ovI.p, S.ovJ.p, W.tkeys.p, S.row_ptr.p, S.col.p,
                                                            S.upidx.p));
  if (npt) KLAUNCH(K_SH, s, k_pair_ov<<<nblk(npt, 256), 256, 0, s>>>(npt, W.bp_pt.p, nov, S.ovI.p, S.ovJ.p, S.pt_ov.p));
  if (nee) KLAUNCH(K_SH, s, k_pair_ov<<<nblk(nee, 256), 256, 0, s>>>(nee, W.bp_ee.p, nov, S.ovI.p, S.ovJ.p, S.ee_ov.p));
  // vertex-ground pairs with the scaled threshold (col_set.cpp:49-63)
  Params Pg = P;
  Pg.dhat = Q.thr;
  vg_pairs(g, Pg, cs, S, s);
  CK(cudaStreamSynchronize(s));
}

void sh_bound(const Geo& g, const Params& P, const ShParams& H, const PairSet& cur, ShScratch& W, CullScratch& cs,
              double* toi, cudaStream_t s) {
  launch_project(g, 2, 1.0, s);
  launch_project(g, 3, 0.0, s);
  const int nk = 2 * g.ns;
  cs.toi_key.ensure(nk);
  double one = 1.0;
  unsigned long long b1;
  memcpy(&b1, &one, sizeof(b1));
  KLAUNCH(K_SH, s, k_fill_key<<<nblk(nk, 256), 256, 0, s>>>(cs.toi_key.p, nk, b1 | 0x8000000000000000ull));
  if (H.full_ccd) {
    if (P.ground && g.nv) launch_vg_toi(g, P, cs.toi_key.p, s);
    ShQuery Q;
    Q.G = grid_of(H);
    Q.qd = 0.0;
    Q.thr = 0.0;
    Q.marg = 0.0;
    Q.traj = 1;
    Q.fix_edge = H.fix_edge;
    if (P.pt && g.nv && g.nf) {
      sh_register(g, H, 0, g.nv, 1, W.tab, s);
      Q.keys = W.tab.keys.p;
      Q.bstart = W.tab.bstart.p;
      Q.bend = W.tab.bend.p;
      KLAUNCH(K_SH, s, k_pt_query<2><<<nblk(g.nf, 128), 128, 0, s>>>(g, Q, nullptr, nullptr, cs.toi_key.p, nullptr));
    }
    if (P.ee && g.ne) {
      sh_register(g, H, 1, g.ne, 1, W.tab, s);
      Q.keys = W.tab.keys.p;
      Q.bstart = W.tab.bstart.p;
      Q.bend = W.tab.bend.p;
      KLAUNCH(K_SH, s, k_ee_query<2><<<nblk(g.ne, 128), 128, 0, s>>>(g, Q, nullptr, nullptr, cs.toi_key.p, nullptr));
    }
  } else {
    KLAUNCH(K_SH, s, k_norm1_bound<<<g.ns, 256, 0, s>>>(g.sc_beg, g.sc_end, g.dq, P.d_sqrt / 2.0, H.safe_factor,
                                                        cs.toi_key.p));
    if (cur.nvg) KLAUNCH(K_SH, s, k_vg_pair_toi<<<nblk(cur.nvg, 256), 256, 0, s>>>(g, P, cur.nvg, cur.vg.p, cs.toi_key.p + 1));
    long long np = (long long)cur.npt + cur.nee;
    if (np) KLAUNCH(K_SH, s, k_pair_toi<<<nblk(np, 128), 128, 0, s>>>(g, cur.npt, cur.pt.p, cur.nee, cur.ee.p, cs.toi_key.p));
  }
  if (!W.h_toi_cap || W.h_toi_cap < nk) {
    if (W.h_toi) CK(cudaFreeHost(W.h_toi));
    CK(cudaMallocHost(&W.h_toi, nk * sizeof(unsigned long long)));
    W.h_toi_cap = nk;
  }
  CK(cudaMemcpyAsync(W.h_toi, cs.toi_key.p, nk * sizeof(unsigned long long), cudaMemcpyDeviceToHost, s));
  CK(cudaStreamSynchronize(s));
  for (int sc = 0; sc < g.ns; ++sc)
    toi[sc] = std::min(key_to_double_h(W.h_toi[2 * sc]), key_to_double_h(W.h_toi[2 * sc + 1]));
}

}  // namespace abd
