// CPU oracle — test infrastructure only. Nothing in the product links, imports or
// executes this file; tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
// use it as the checker and as the timed CPU port of the reference.
//
// A plain C++17 + OpenMP restatement of the reference's per-frame step
// `ABD::implicit_euler` (model/abd.cpp:30-140) with its iAABB culling
// (model/iaabb.cpp, model/thread_local_culling.cpp), per-pair IPC terms
// (model/core_ipc.cpp, pt_ipc.cpp, ee_ipc.cpp, vg_ipc.cpp, psd.h, friction.cpp),
// block-sparse assembly (model/assemble_matrices.cpp, sparse.cpp), inertia and
// orthogonality (model/mutils.cpp, othogonal_energy.cpp), a direct block-sparse
// Cholesky standing in for Pardiso LLT (abd.cpp:229-303), CCD (model/collision.cpp)
// and the Armijo line search (model/line_search.cpp, energy.cpp).
// The narrow phase is the brute-force path of thread_local_culling.cpp (the BVH branch
// the reference takes above `thres` primitives stores float node bounds and can drop
// borderline candidates; the canonical pair set here is the brute-force one).
#include <omp.h>

#include <array>
#include <cstdint>
#include <cstdio>
#include <map>
#include <set>
#include <unordered_map>
#include <vector>

#include "oracle_ipc.h"

namespace orc {

struct Config {
  // doubles
  double dt, kappa, dhat, ortho_kappa, ground_offset, mu, evh, eps_x, backoff, c1, tol, max_uk, dq_tol,
      gravity_y, ls_grad_tol;
  // ints
  int max_iter, ground, pt, ee, psd, line_search, upper_bound, vg_fric, pt_fric, ee_fric, clip, n_threads;
  // broad-phase selection and spatial hashing ("iaabb", "full_ccd", "safe_factor",
  // "spatial hashing" {min_xyz, dx, xyz_bits}; view/control.cpp:37-68)
  double safe_factor, sh_min_xyz, sh_dx;
  int iaabb, full_ccd, sh_bits, sh_fix_edge;
  // "damping": {enable, alpha, beta} (view/control.cpp:35, 60-61)
  int damp;
  double damp_alpha, damp_beta;
  // Newton iterations per frame at most (0: unbounded, the reference's loop); a library
  // option for frames whose lagged-friction iteration cycles
  int max_iter_frame;
};

struct I4 {
  int v[4];
  int operator[](int i) const { return v[i]; }
};

struct Overlap {
  int I, J;
  Box cull;
};

struct PairSet {
  std::vector<Overlap> ov;
  std::vector<int> pt_off, ee_off;  // per overlap ranges into pt / ee (size nov+1)
  std::vector<I4> pt, ee;
  std::vector<int8_t> pt_ty, ee_ty;
  std::vector<std::array<int, 2>> vg;
};

struct Body {
  double q[12], q0[12], dqdt[12], dq[12];
  double mass, Ic;
  int v_off, nv, e_off, ne, f_off, nf;
  Box rest;  // rest AABB inflated by sqrt(dhat)  (iaabb.cpp:23-39)
  double grad[12];
  M12 hess;
};

struct Stats {
  int newton_iters, ls_trials, n_pt, n_ee, n_vg, status;
  double toi_min, alpha_min, t_ipc, t_solver, t_ccd, t_ls;
};

enum { ST_OK = 0, ST_NAN = 1, ST_LS_STALL = 2, ST_TOI_TINY = 4, ST_NOT_SPD = 5, ST_SAME_DIR = 10 };

struct Scene {
  Config cfg;
  BarrierParams bp;
  FrictionParams fp;
  double d_sqrt;
  std::vector<Body> b;
  std::vector<double> rest;  // 3 * nv
  std::vector<int> edges;    // 2 * ne (local vertex ids)
  std::vector<int> faces;    // 3 * nf (local vertex ids)
  std::vector<V3> X;         // v_transformed
  std::vector<V3> Xq;        // positions at q (vt1_buffer)
  std::vector<V3> X0;        // positions at q0
  int iter = 0;              // cumulative Newton counter (abd.h:53, never reset per frame)
  int g_cnt = 0, p_cnt = 0;  // consecutive tiny-TOI counters (iaabb.cpp:302-313, 533-540)
  std::vector<double> lastdq;  // previous Newton step, kept across frames (abd.h member)
  PairSet set;
  std::vector<Mat<2, 12>> pt_tk, ee_tk;
  std::vector<double> pt_lam, ee_lam, g_lam;
  Stats st;
  int nv_tot = 0;
};

// ---------------------------------------------------------------------------------
// Vertex projection x = A xbar + p (affine_body.h:34-98): row r is
// ((a1_r x0 + a2_r x1) + a3_r x2) + p_r with a_k = q[3k .. 3k+2].
static inline V3 project_pt(const double* q, const double* xr) {
  V3 o;
  for (int r = 0; r < 3; ++r) o[r] = ((q[3 + r] * xr[0] + q[6 + r] * xr[1]) + q[9 + r] * xr[2]) + q[r];
  return o;
}
static inline void q_plus(const double* q, const double* dq, double* out) {
  for (int i = 0; i < 12; ++i) out[i] = q[i] + dq[i];
}

// iaabb.cpp:40-72: transformed AABB of the inflated rest box.
static Box affine_box(const Box& r, const double* q) {
  V3 lo, hi;
  bool first = true;
  for (int i = 0; i < 2; ++i)
    for (int j = 0; j < 2; ++j)
      for (int k = 0; k < 2; ++k) {
        double c[3] = {i ? r.hi.x : r.lo.x, j ? r.hi.y : r.lo.y, k ? r.hi.z : r.lo.z};
        V3 p;
        for (int row = 0; row < 3; ++row) p[row] = (q[3 + row] * c[0] + q[6 + row] * c[1]) + q[9 + row] * c[2];
        if (first) { lo = hi = p; first = false; }
        else { lo = vmin(lo, p); hi = vmax(hi, p); }
      }
  V3 t(q[0], q[1], q[2]);
  return Box{lo + t, hi + t};
}

static void project_all(Scene& s, int which) {
  // which: 0 -> q0 (X0), 1 -> q (Xq and X), 2 -> q + dq (X)
  int nb = (int)s.b.size();
#pragma omp parallel for schedule(static)
  for (int I = 0; I < nb; ++I) {
    Body& c = s.b[I];
    double qq[12];
    const double* q = c.q;
    if (which == 0) q = c.q0;
    if (which == 2) { q_plus(c.q, c.dq, qq); q = qq; }
    for (int v = 0; v < c.nv; ++v) {
      V3 x = project_pt(q, &s.rest[3 * (c.v_off + v)]);
      if (which == 0) s.X0[c.v_off + v] = x;
      else if (which == 1) { s.Xq[c.v_off + v] = x; s.X[c.v_off + v] = x; }
      else s.X[c.v_off + v] = x;
    }
  }
}

// ---------------------------------------------------------------------------------
// Broad phase (iaabb.cpp:98-202): body boxes at q (vtn 1), q + dq (vtn 2) or the union
// of both (vtn 3); every pair whose boxes overlap on all axes, with the intersection box.
static void body_overlaps(Scene& s, int vtn, std::vector<Overlap>& ov) {
  int nb = (int)s.b.size();
  std::vector<Box> bb(nb);
  for (int I = 0; I < nb; ++I) {
    Body& c = s.b[I];
    double qq[12];
    q_plus(c.q, c.dq, qq);
    if (vtn == 1) bb[I] = affine_box(c.rest, c.q);
    else if (vtn == 2) bb[I] = affine_box(c.rest, qq);
    else bb[I] = merge(affine_box(c.rest, c.q), affine_box(c.rest, qq));
  }
  ov.clear();
  std::vector<std::vector<Overlap>> rows(nb);
#pragma omp parallel for schedule(dynamic, 8)
  for (int I = 0; I < nb; ++I)
    for (int J = I + 1; J < nb; ++J) {
      Box cull;
      if (intersection(bb[I], bb[J], cull)) rows[I].push_back(Overlap{I, J, cull});
    }
  for (int I = 0; I < nb; ++I) ov.insert(ov.end(), rows[I].begin(), rows[I].end());
}

struct Lists {
  std::vector<int> vi, vj, ei, ej, fi, fj;
};

static inline V3 Xat(const Scene& s, int body, int v) { return s.X[s.b[body].v_off + v]; }
static inline V3 Xqat(const Scene& s, int body, int v) { return s.Xq[s.b[body].v_off + v]; }
static inline void edge_at(const Scene& s, const std::vector<V3>& P, int body, int e, V3 out[2]) {
  const Body& c = s.b[body];
  const int* ed = &s.edges[2 * (c.e_off + e)];
  out[0] = P[c.v_off + ed[0]];
  out[1] = P[c.v_off + ed[1]];
}
static inline void face_at(const Scene& s, const std::vector<V3>& P, int body, int f, V3 out[3]) {
  const Body& c = s.b[body];
  const int* fc = &s.faces[3 * (c.f_off + f)];
  out[0] = P[c.v_off + fc[0]];
  out[1] = P[c.v_off + fc[1]];
  out[2] = P[c.v_off + fc[2]];
}

// Primitive binning (iaabb.cpp:315-443): vertices, edges and faces of each body that
// touch the overlap's cull box, per side of the merged (I, J) overlap.
static void bin_side(const Scene& s, int body, const Box& cull, bool traj, std::vector<int>& v,
                     std::vector<int>& e, std::vector<int>& f) {
  const Body& c = s.b[body];
  for (int k = 0; k < c.nv; ++k) {
    V3 p = Xat(s, body, k);
    Box a = traj ? box_of(p, Xqat(s, body, k)) : Box{p, p};
    if (intersects(cull, a)) v.push_back(k);
  }
  for (int k = 0; k < c.ne; ++k) {
    V3 e1[2], e0[2];
    edge_at(s, s.X, body, k, e1);
    Box a;
    if (traj) {
      edge_at(s, s.Xq, body, k, e0);
      a = box_of4(e1[0], e1[1], e0[0], e0[1]);
    } else {
      a = box_of(e1[0], e1[1]);
    }
    if (intersects(cull, a)) e.push_back(k);
  }
  for (int k = 0; k < c.nf; ++k) {
    V3 f1[3], f0[3];
    face_at(s, s.X, body, k, f1);
    Box a = box_of(f1[0], f1[1], f1[2]);
    if (traj) {
      face_at(s, s.Xq, body, k, f0);
      a = merge(box_of(f0[0], f0[1], f0[2]), a);
    }
    if (intersects(a, cull)) f.push_back(k);
  }
}

// vf_col_set / ee_col_set brute-force branches (thread_local_culling.cpp:209-386).
static void pt_narrow(const Scene& s, const std::vector<int>& vl, const std::vector<int>& fl, int I, int J,
                      std::vector<I4>& out, std::vector<int8_t>& ty) {
  double ds = s.d_sqrt;
  for (int vi : vl) {
    V3 v = Xat(s, I, vi);
    Box bv{V3(v.x - ds, v.y - ds, v.z - ds), V3(v.x + ds, v.y + ds, v.z + ds)};
    for (int fj : fl) {
      V3 f[3];
      face_at(s, s.X, J, fj, f);
      Box bf = box_of(f[0], f[1], f[2]);
      if (!intersects(bv, bf)) continue;
      PTType t = pt_type(v, f[0], f[1], f[2]);
      double d = pt_dist(v, f[0], f[1], f[2], t);
      if (d < s.bp.dhat) {
        out.push_back(I4{{I, vi, J, fj}});
        ty.push_back((int8_t)t);
      }
    }
  }
}
static void ee_narrow(const Scene& s, const std::vector<int>& el, const std::vector<int>& fl, int I, int J,
                      std::vector<I4>& out, std::vector<int8_t>& ty) {
  double ds = s.d_sqrt;
  for (int ei : el) {
    V3 a[2];
    edge_at(s, s.X, I, ei, a);
    Box ba = inflate(box_of(a[0], a[1]), ds);
    for (int ej : fl) {
      V3 b[2];
      edge_at(s, s.X, J, ej, b);
      Box bb = box_of(b[0], b[1]);
      if (!intersects(ba, bb)) continue;
      EEType t = ee_type(a[0], a[1], b[0], b[1]);
      double d = ee_dist(a[0], a[1], b[0], b[1], t);
      if (d < s.bp.dhat) {
        out.push_back(I4{{I, ei, J, ej}});
        ty.push_back((int8_t)t);
      }
    }
  }
}

// vf_col_time / ee_col_time brute-force branches (thread_local_culling.cpp:28-207).
static double pt_traj(const Scene& s, const std::vector<int>& vl, const std::vector<int>& fl, int I, int J) {
  double toi = 1.0;
  for (int vi : vl) {
    V3 v1 = Xat(s, I, vi), v0 = Xqat(s, I, vi);
    Box bv = box_of(v0, v1);
    for (int fj : fl) {
      V3 f1[3], f0[3];
      face_at(s, s.X, J, fj, f1);
      face_at(s, s.Xq, J, fj, f0);
      Box bf = merge(box_of(f0[0], f0[1], f0[2]), box_of(f1[0], f1[1], f1[2]));
      if (!intersects(bv, bf)) continue;
      toi = std::min(toi, pt_collision_time(v0, f0, v1, f1));
    }
  }
  return toi;
}
static double ee_traj(const Scene& s, const std::vector<int>& el, const std::vector<int>& fl, int I, int J) {
  double toi = 1.0;
  for (int ei : el) {
    V3 a1[2], a0[2];
    edge_at(s, s.X, I, ei, a1);
    edge_at(s, s.Xq, I, ei, a0);
    Box ba = box_of4(a0[0], a0[1], a1[0], a1[1]);
    for (int ej : fl) {
      V3 b1[2], b0[2];
      edge_at(s, s.X, J, ej, b1);
      edge_at(s, s.Xq, J, ej, b0);
      Box bb = box_of4(b0[0], b0[1], b1[0], b1[1]);
      if (!intersects(ba, bb)) continue;
      toi = std::min(toi, ee_collision_time(a0, b0, a1, b1));
    }
  }
  return toi;
}

// IAABB::iaabb_brute_force (iaabb.cpp:545-568). vtn 1/2 fill `out`; vtn 3 returns the
// time of impact of the trajectory q -> q + dq (1.0 if none).
static double iaabb(Scene& s, int vtn, PairSet* out) {
  bool traj = vtn == 3;
  project_all(s, vtn == 1 ? 1 : 2);
  if (traj) {
    // vt1_buffer at q (iaabb.cpp:446-468)
    int nb = (int)s.b.size();
#pragma omp parallel for schedule(static)
    for (int I = 0; I < nb; ++I) {
      Body& c = s.b[I];
      for (int v = 0; v < c.nv; ++v) s.Xq[c.v_off + v] = project_pt(c.q, &s.rest[3 * (c.v_off + v)]);
    }
  }
  std::vector<Overlap> ov;
  body_overlaps(s, vtn, ov);
  int nov = (int)ov.size();
  double toi_g = 1.0;
  std::vector<std::array<int, 2>> vg;
  if (s.cfg.ground) {
    for (int I = 0; I < (int)s.b.size(); ++I) {
      Body& c = s.b[I];
      for (int v = 0; v < c.nv; ++v) {
        V3 p = s.X[c.v_off + v];
        if (!traj) {
          double d = p.y + s.cfg.ground_offset;
          d = d * d;
          if (d < s.bp.dhat) vg.push_back({I, v});
        } else {
          // collision.cpp:83-105
          double d2 = p.y + s.cfg.ground_offset;
          if (d2 < 0) {
            double d1 = s.Xq[c.v_off + v].y + s.cfg.ground_offset;
            double t = d1 / (d1 - d2);
            toi_g = std::min(toi_g, t);
          }
        }
      }
    }
  }
  std::vector<std::vector<I4>> pt(nov), ee(nov);
  std::vector<std::vector<int8_t>> ptt(nov), eet(nov);
  std::vector<double> tois(nov, 1.0);
#pragma omp parallel for schedule(dynamic, 1)
  for (int o = 0; o < nov; ++o) {
    Lists L;
    bin_side(s, ov[o].I, ov[o].cull, traj, L.vi, L.ei, L.fi);
    bin_side(s, ov[o].J, ov[o].cull, traj, L.vj, L.ej, L.fj);
    int I = ov[o].I, J = ov[o].J;
    if (!traj) {
      ee_narrow(s, L.ei, L.ej, I, J, ee[o], eet[o]);
      pt_narrow(s, L.vi, L.fj, I, J, pt[o], ptt[o]);
      pt_narrow(s, L.vj, L.fi, J, I, pt[o], ptt[o]);
    } else {
      double t1 = pt_traj(s, L.vi, L.fj, I, J);
      double t2 = pt_traj(s, L.vj, L.fi, J, I);
      double t3 = ee_traj(s, L.ei, L.ej, I, J);
      tois[o] = std::min(t1, std::min(t2, t3));
    }
  }
  if (traj) {
    double toi_p = 1.0;
    for (int o = 0; o < nov; ++o) toi_p = std::min(toi_p, tois[o]);
    if (s.cfg.ground) {
      if (toi_g < 1e-6) s.g_cnt++; else s.g_cnt = 0;
    }
    if (toi_p < 1e-6) s.p_cnt++; else s.p_cnt = 0;
    return std::min(toi_g, toi_p);
  }
  PairSet& P = *out;
  P.ov = ov;
  P.pt.clear(); P.ee.clear(); P.pt_ty.clear(); P.ee_ty.clear();
  P.pt_off.assign(nov + 1, 0);
  P.ee_off.assign(nov + 1, 0);
  for (int o = 0; o < nov; ++o) {
    P.pt_off[o] = (int)P.pt.size();
    P.ee_off[o] = (int)P.ee.size();
    P.pt.insert(P.pt.end(), pt[o].begin(), pt[o].end());
    P.pt_ty.insert(P.pt_ty.end(), ptt[o].begin(), ptt[o].end());
    P.ee.insert(P.ee.end(), ee[o].begin(), ee[o].end());
    P.ee_ty.insert(P.ee_ty.end(), eet[o].begin(), eet[o].end());
  }
  P.pt_off[nov] = (int)P.pt.size();
  P.ee_off[nov] = (int)P.ee.size();
  P.vg = vg;
  return 1.0;
}

// ---------------------------------------------------------------------------------
// Spatial-hash broad phase (iaabb even): spatial_hashing.cpp:11-211 and the global-list
// branches of gen_collision_set (col_set.cpp:20-339) and step_size_upper_bound
// (upper_bound.cpp:16-277). Cells are tovec3i(x) = int(max(x - min_xyz, 0) / dx) per
// axis; a cell's bucket keeps the low xyz_bits bits of each axis (hash(), :11-21), so
// cells that agree modulo 2^bits share a bucket. Buckets here are unbounded (the
// reference keeps n_buffer entries per bucket and logs an error beyond that).
struct SHash {
  int bits;
  double min_xyz, dx;
  std::vector<std::vector<int>> bucket;  // entries: (body << 16) | pid, as Primitive::as_uint
  SHash(int b, double mn, double d) : bits(b), min_xyz(mn), dx(d), bucket(size_t(1) << (3 * b)) {}
  int cell(double f) const { return (int)(std::max(f - min_xyz, 0.0) / dx); }
  int hash(int i, int j, int k) const {
    int m = (1 << bits) - 1;
    return (((i & m) << bits | (j & m)) << bits) | (k & m);
  }
  void reg(const V3& lo, const V3& hi, int body, int pid) {
    int l[3] = {cell(lo.x), cell(lo.y), cell(lo.z)}, u[3] = {cell(hi.x), cell(hi.y), cell(hi.z)};
    for (int i = l[0]; i <= u[0]; ++i)
      for (int j = l[1]; j <= u[1]; ++j)
        for (int k = l[2]; k <= u[2]; ++k) bucket[hash(i, j, k)].push_back((body << 16) | pid);
  }
  // query_interval (:71-113): entries of every bucket the cell range touches, other
  // bodies only, sorted and unique.
  void query(const V3& lo, const V3& hi, int body_exl, std::vector<int>& out) const {
    out.clear();
    int l[3] = {cell(lo.x), cell(lo.y), cell(lo.z)}, u[3] = {cell(hi.x), cell(hi.y), cell(hi.z)};
    for (int i = l[0]; i <= u[0]; ++i)
      for (int j = l[1]; j <= u[1]; ++j)
        for (int k = l[2]; k <= u[2]; ++k)
          for (int e : bucket[hash(i, j, k)])
            if ((e >> 16) != body_exl) out.push_back(e);
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
  }
};

static inline V3 vadd(const V3& a, double d) { return V3(a.x + d, a.y + d, a.z + d); }

// Orders a pair set the way the overlap-based paths store it: overlaps (I < J) sorted,
// and per overlap the PT pairs with the vertex on I, then on J, then the EE pairs, each
// by (primitive of the first body, primitive of the second). The reference's spatial-hash
// path appends the pairs of its OpenMP threads in scheduling order, so only the set is
// defined there.
static void canonical_set(const std::vector<I4>& pt, const std::vector<int8_t>& ptt, const std::vector<I4>& ee,
                          const std::vector<int8_t>& eet, PairSet& P) {
  struct K {
    long long key;
    int src;
  };
  auto pt_key = [](const I4& p) {
    int A = p[0], B = p[2];
    long long lo = std::min(A, B), hi = std::max(A, B), sub = A < B ? 0 : 1;
    return (lo << 47) | (hi << 32) | (sub << 30) | ((long long)p[1] << 15) | (long long)p[3];
  };
  auto ee_key = [](const I4& p) {
    return ((long long)p[0] << 47) | ((long long)p[2] << 32) | (2ll << 30) | ((long long)p[1] << 15) | (long long)p[3];
  };
  std::vector<K> kp(pt.size()), ke(ee.size());
  for (size_t k = 0; k < pt.size(); ++k) kp[k] = K{pt_key(pt[k]), (int)k};
  for (size_t k = 0; k < ee.size(); ++k) ke[k] = K{ee_key(ee[k]), (int)k};
  auto cmp = [](const K& a, const K& b) { return a.key < b.key; };
  std::sort(kp.begin(), kp.end(), cmp);
  std::sort(ke.begin(), ke.end(), cmp);
  std::vector<long long> bp;
  for (auto& k : kp) bp.push_back(k.key >> 32);
  for (auto& k : ke) bp.push_back(k.key >> 32);
  std::sort(bp.begin(), bp.end());
  bp.erase(std::unique(bp.begin(), bp.end()), bp.end());
  int nov = (int)bp.size();
  P.ov.assign(nov, Overlap{});
  for (int o = 0; o < nov; ++o) {
    P.ov[o].I = (int)(bp[o] >> 15);
    P.ov[o].J = (int)(bp[o] & 0x7fff);
  }
  P.pt.clear(); P.ee.clear(); P.pt_ty.clear(); P.ee_ty.clear();
  P.pt_off.assign(nov + 1, 0);
  P.ee_off.assign(nov + 1, 0);
  size_t a = 0, b = 0;
  for (int o = 0; o < nov; ++o) {
    P.pt_off[o] = (int)P.pt.size();
    P.ee_off[o] = (int)P.ee.size();
    for (; a < kp.size() && (kp[a].key >> 32) == bp[o]; ++a) {
      P.pt.push_back(pt[kp[a].src]);
      P.pt_ty.push_back(ptt[kp[a].src]);
    }
    for (; b < ke.size() && (ke[b].key >> 32) == bp[o]; ++b) {
      P.ee.push_back(ee[ke[b].src]);
      P.ee_ty.push_back(eet[ke[b].src]);
    }
  }
  P.pt_off[nov] = (int)P.pt.size();
  P.ee_off[nov] = (int)P.ee.size();
}

// gen_collision_set (col_set.cpp:20-339), global point / edge / triangle lists.
static void sh_collision_set(Scene& s, bool vt2, PairSet* out) {
  project_all(s, vt2 ? 2 : 1);
  const double sf = s.cfg.safe_factor;
  const double thr = s.bp.dhat * (sf * sf);
  const double qd = s.d_sqrt * sf;
  int nb = (int)s.b.size();
  std::vector<std::array<int, 2>> vg;
  if (s.cfg.ground)
    for (int I = 0; I < nb; ++I)
      for (int v = 0; v < s.b[I].nv; ++v) {
        double d = Xat(s, I, v).y + s.cfg.ground_offset;
        d = d * d;
        if (d < thr) vg.push_back({I, v});
      }
  std::vector<I4> pt, ee;
  std::vector<int8_t> ptt, eet;
  std::vector<int> cand;
  if (s.cfg.pt) {
    SHash h(s.cfg.sh_bits, s.cfg.sh_min_xyz, s.cfg.sh_dx);
    for (int I = 0; I < nb; ++I)
      for (int v = 0; v < s.b[I].nv; ++v) {
        V3 p = Xat(s, I, v);
        h.reg(p, p, I, v);
      }
    for (int J = 0; J < nb; ++J)
      for (int f = 0; f < s.b[J].nf; ++f) {
        V3 t[3];
        face_at(s, s.X, J, f, t);
        V3 lo = vmin(vmin(t[0], t[1]), t[2]), hi = vmax(vmax(t[0], t[1]), t[2]);
        h.query(vadd(lo, -qd), vadd(hi, qd), J, cand);
        for (int e : cand) {
          int I = e >> 16, v = e & 0xffff;
          V3 p = Xat(s, I, v);
          PTType ty = pt_type(p, t[0], t[1], t[2]);
          double d = pt_dist(p, t[0], t[1], t[2], ty);
          if (d < thr) {
            pt.push_back(I4{{I, v, J, f}});
            ptt.push_back((int8_t)ty);
          }
        }
      }
  }
  if (s.cfg.ee) {
    SHash h(s.cfg.sh_bits, s.cfg.sh_min_xyz, s.cfg.sh_dx);
    for (int I = 0; I < nb; ++I)
      for (int e = 0; e < s.b[I].ne; ++e) {
        V3 a[2];
        edge_at(s, s.X, I, e, a);
        h.reg(vmin(a[0], a[1]), vmax(a[0], a[1]), I, e);
      }
    for (int J = 0; J < nb; ++J)
      for (int ej = 0; ej < s.b[J].ne; ++ej) {
        V3 b2[2];
        edge_at(s, s.X, J, ej, b2);
        h.query(vadd(vmin(b2[0], b2[1]), -qd), vadd(vmax(b2[0], b2[1]), qd), J, cand);
        for (int e : cand) {
          int I = e >> 16, ei = e & 0xffff;
          if (I > J) continue;
          V3 a[2];
          edge_at(s, s.X, I, ei, a);
          EEType ty = ee_type(a[0], a[1], b2[0], b2[1]);
          double d = ee_dist(a[0], a[1], b2[0], b2[1], ty);
          if (d < thr) {
            ee.push_back(I4{{I, ei, J, ej}});
            eet.push_back((int8_t)ty);
          }
        }
      }
  }
  canonical_set(pt, ptt, ee, eet, *out);
  out->vg = vg;
}

// step_size_upper_bound (upper_bound.cpp:16-277). With full_ccd the trajectories are
// hashed (vertex trajectories as segments; edge trajectories, as in the reference,
// registered by their start position only unless sh_fix_edge is set) and every candidate
// that shares a bucket gets an exact time of impact; otherwise the bound is
// d_sqrt / 2 / max_I |dq_I|_1 * safe_factor, lowered by the TOIs of the current pairs.
static double sh_upper_bound(Scene& s) {
  int nb = (int)s.b.size();
  project_all(s, 2);
  for (int I = 0; I < nb; ++I) {
    Body& c = s.b[I];
    for (int v = 0; v < c.nv; ++v) s.Xq[c.v_off + v] = project_pt(c.q, &s.rest[3 * (c.v_off + v)]);
  }
  auto ground_t = [&](int I, int v) {
    double d2 = Xat(s, I, v).y + s.cfg.ground_offset;
    if (!(d2 < 0)) return 1.0;
    double d1 = Xqat(s, I, v).y + s.cfg.ground_offset;
    return d1 / (d1 - d2);
  };
  double toi = 1.0;
  std::vector<int> cand;
  if (s.cfg.full_ccd) {
    if (s.cfg.ground)
      for (int I = 0; I < nb; ++I)
        for (int v = 0; v < s.b[I].nv; ++v) toi = std::min(toi, ground_t(I, v));
    if (s.cfg.pt) {
      SHash h(s.cfg.sh_bits, s.cfg.sh_min_xyz, s.cfg.sh_dx);
      for (int I = 0; I < nb; ++I)
        for (int v = 0; v < s.b[I].nv; ++v) {
          V3 p0 = Xqat(s, I, v), p1 = Xat(s, I, v);
          h.reg(vmin(p0, p1), vmax(p0, p1), I, v);
        }
      for (int J = 0; J < nb; ++J)
        for (int f = 0; f < s.b[J].nf; ++f) {
          V3 f0[3], f1[3];
          face_at(s, s.Xq, J, f, f0);
          face_at(s, s.X, J, f, f1);
          V3 lo = vmin(vmin(vmin(f0[0], f0[1]), f0[2]), vmin(vmin(f1[0], f1[1]), f1[2]));
          V3 hi = vmax(vmax(vmax(f0[0], f0[1]), f0[2]), vmax(vmax(f1[0], f1[1]), f1[2]));
          h.query(lo, hi, J, cand);
          for (int e : cand) {
            int I = e >> 16, v = e & 0xffff;
            toi = std::min(toi, pt_collision_time(Xqat(s, I, v), f0, Xat(s, I, v), f1));
          }
        }
    }
    if (s.cfg.ee) {
      SHash h(s.cfg.sh_bits, s.cfg.sh_min_xyz, s.cfg.sh_dx);
      for (int I = 0; I < nb; ++I)
        for (int e = 0; e < s.b[I].ne; ++e) {
          V3 a0[2], a1[2];
          edge_at(s, s.Xq, I, e, a0);
          edge_at(s, s.X, I, e, a1);
          V3 lo = vmin(a0[0], a0[1]), hi = vmax(a0[0], a0[1]);
          if (s.cfg.sh_fix_edge) {
            lo = vmin(lo, vmin(a1[0], a1[1]));
            hi = vmax(hi, vmax(a1[0], a1[1]));
          }
          h.reg(lo, hi, I, e);
        }
      for (int J = 0; J < nb; ++J)
        for (int ej = 0; ej < s.b[J].ne; ++ej) {
          V3 b0[2], b1[2];
          edge_at(s, s.Xq, J, ej, b0);
          edge_at(s, s.X, J, ej, b1);
          V3 lo = vmin(vmin(b0[0], b0[1]), vmin(b1[0], b1[1])), hi = vmax(vmax(b0[0], b0[1]), vmax(b1[0], b1[1]));
          h.query(lo, hi, J, cand);
          for (int e : cand) {
            int I = e >> 16, ei = e & 0xffff;
            if (I > J) continue;
            V3 a0[2], a1[2];
            edge_at(s, s.Xq, I, ei, a0);
            edge_at(s, s.X, I, ei, a1);
            toi = std::min(toi, ee_collision_time(a0, b0, a1, b1));
          }
        }
    }
    return toi;
  }
  double n1 = 0.0;
  for (int I = 0; I < nb; ++I) {
    double a = 0.0;
    for (int i = 0; i < 12; ++i) a += std::fabs(s.b[I].dq[i]);
    n1 = std::max(n1, a);
  }
  toi = s.d_sqrt / 2.0 / n1 * s.cfg.safe_factor;
  toi = std::min(1.0, toi);
  const PairSet& P = s.set;
  for (auto& v : P.vg) toi = std::min(toi, ground_t(v[0], v[1]));
  for (auto& p : P.pt) {
    V3 f0[3], f1[3];
    face_at(s, s.Xq, p[2], p[3], f0);
    face_at(s, s.X, p[2], p[3], f1);
    toi = std::min(toi, pt_collision_time(Xqat(s, p[0], p[1]), f0, Xat(s, p[0], p[1]), f1));
  }
  for (auto& p : P.ee) {
    V3 a0[2], a1[2], b0[2], b1[2];
    edge_at(s, s.Xq, p[0], p[1], a0);
    edge_at(s, s.X, p[0], p[1], a1);
    edge_at(s, s.Xq, p[2], p[3], b0);
    edge_at(s, s.X, p[2], p[3], b1);
    toi = std::min(toi, ee_collision_time(a0, b0, a1, b1));
  }
  return toi;
}

// Culling dispatch (abd.cpp:48-51, 157-174; line_search.cpp:88-110): iaabb odd culls with
// the iAABB brute force, even with the spatial hash; iaabb > 1 bounds the step with the
// iAABB trajectory pass, otherwise with step_size_upper_bound.
static double cull(Scene& s, int vtn, PairSet* out) {
  if (vtn == 3) return s.cfg.iaabb > 1 ? iaabb(s, 3, nullptr) : sh_upper_bound(s);
  if (s.cfg.iaabb % 2) return iaabb(s, vtn, out);
  sh_collision_set(s, vtn == 2, out);
  return 1.0;
}

// ---------------------------------------------------------------------------------
// Inertia and orthogonality (othogonal_energy.cpp:16-62, mutils.cpp:53-76, 197-201, 245-252).
static void ortho_grad(const double* q, double kappa, double* g) {
  for (int i = 0; i < 12; ++i) g[i] = 0;
  for (int i = 1; i < 4; ++i) {
    V3 acc;
    V3 qi(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
    for (int j = 1; j < 4; ++j) {
      V3 qj(q[3 * j], q[3 * j + 1], q[3 * j + 2]);
      acc = acc + (dot(qi, qj) - (i == j ? 1.0 : 0.0)) * qj;
    }
    for (int r = 0; r < 3; ++r) g[3 * i + r] = 4 * kappa * acc[r];
  }
}
static void ortho_hess(const double* q, double kappa, M12& H) {
  H = M12();
  V3 a[4];
  for (int i = 0; i < 4; ++i) a[i] = V3(q[3 * i], q[3 * i + 1], q[3 * i + 2]);
  for (int i = 1; i < 4; ++i)
    for (int j = 1; j < 4; ++j) {
      double h[3][3];
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
          if (i == j) {
            double v = 2 * a[i][r] * a[i][c] + (r == c ? (dot(a[i], a[i]) - 1) : 0.0);
            for (int k = 1; k < 4; ++k)
              if (k != i) v += a[k][r] * a[k][c];
            h[r][c] = v;
          } else {
            h[r][c] = (r == c ? dot(a[j], a[i]) : 0.0) + a[j][r] * a[i][c];
          }
        }
      for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) H(3 * i + r, 3 * j + c) = h[r][c] * 4 * kappa;
    }
}
static double ortho_energy(const double* q, double kappa) {
  double E = 0;
  for (int i = 1; i < 4; ++i)
    for (int j = 1; j < 4; ++j) {
      V3 qi(q[3 * i], q[3 * i + 1], q[3 * i + 2]), qj(q[3 * j], q[3 * j + 1], q[3 * j + 2]);
      double e = dot(qi, qj) - (i == j ? 1.0 : 0.0);
      E += e * e;
    }
  return E * kappa;
}
static void q_tilde(const Scene& s, const Body& c, double* qt) {
  double dt = s.cfg.dt;
  for (int i = 0; i < 12; ++i) qt[i] = c.q0[i] + dt * c.dqdt[i];
  qt[1] += dt * dt * s.cfg.gravity_y;
}
static double inertia_energy(const Scene& s, const Body& c, const double* q) {
  if (c.mass < 0.0) return 0.0;
  double qt[12];
  q_tilde(s, c, qt);
  double pp = 0, rr = 0;
  for (int i = 0; i < 3; ++i) pp += (q[i] - qt[i]) * (q[i] - qt[i]);
  for (int i = 3; i < 12; ++i) rr += (q[i] - qt[i]) * (q[i] - qt[i]);
  double dt = s.cfg.dt;
  return ortho_energy(q, s.cfg.ortho_kappa) * dt * dt + 0.5 * (pp * c.mass + rr * c.Ic);
}

// ---------------------------------------------------------------------------------
// Body-space chain rule: x = J(xbar) q with J = [I, x0 I, x1 I, x2 I].
static inline void jac_rows(const double* xr, double J[3][12]) {
  for (int r = 0; r < 3; ++r)
    for (int c = 0; c < 12; ++c) J[r][c] = 0;
  for (int r = 0; r < 3; ++r) {
    J[r][r] = 1;
    J[r][3 + r] = xr[0];
    J[r][6 + r] = xr[1];
    J[r][9 + r] = xr[2];
  }
}

struct OverlapAccum {
  M12 off, dI, dJ;
  double gI[12], gJ[12];
};

// Chains the vertex-space (H, g) of points 0..na-1 on body A and na..3 on body B into
// the body blocks (ipc_term, pt_ipc.cpp:118-186; ipc_term_ee, ee_ipc.cpp:128-210) and
// scatters them (output_hessian_gradient, assemble_matrices.cpp:28-59).
static void chain_scatter(const Scene& s, const M12& H, const V12& g, const double* xr[4], int na, int A, int B,
                          OverlapAccum& acc, bool a_is_I) {
  double JA[12][12] = {}, JB[12][12] = {};  // rows: vertex dofs of each side
  int nA = 3 * na, nB = 12 - nA;
  for (int i = 0; i < 4; ++i) {
    double Jr[3][12];
    jac_rows(xr[i], Jr);
    for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 12; ++c) {
        if (i < na) JA[3 * i + r][c] = Jr[r][c];
        else JB[3 * (i - na) + r][c] = Jr[r][c];
      }
  }
  M12 hA, hB, off;
  double gA[12] = {}, gB[12] = {};
  // hA = JA^T H_AA JA, hB = JB^T H_BB JB, off = JA^T H_AB JB
  for (int p = 0; p < 12; ++p)
    for (int q = 0; q < 12; ++q) {
      double sa = 0, sb = 0, so = 0;
      for (int i = 0; i < nA; ++i)
        for (int j = 0; j < nA; ++j) sa += JA[i][p] * H(i, j) * JA[j][q];
      for (int i = 0; i < nB; ++i)
        for (int j = 0; j < nB; ++j) sb += JB[i][p] * H(nA + i, nA + j) * JB[j][q];
      for (int i = 0; i < nA; ++i)
        for (int j = 0; j < nB; ++j) so += JA[i][p] * H(i, nA + j) * JB[j][q];
      hA(p, q) = sa;
      hB(p, q) = sb;
      off(p, q) = so;
    }
  for (int p = 0; p < 12; ++p) {
    for (int i = 0; i < nA; ++i) gA[p] += JA[i][p] * g(i, 0);
    for (int i = 0; i < nB; ++i) gB[p] += JB[i][p] * g(nA + i, 0);
  }
  bool a_dyn = s.b[A].mass > 0.0, b_dyn = s.b[B].mass > 0.0;
  M12& dA = a_is_I ? acc.dI : acc.dJ;
  M12& dB = a_is_I ? acc.dJ : acc.dI;
  double* grA = a_is_I ? acc.gI : acc.gJ;
  double* grB = a_is_I ? acc.gJ : acc.gI;
  if (b_dyn) {
    if (a_dyn) {
      // block (A, B) += off; stored as block (I, J)
      for (int p = 0; p < 12; ++p)
        for (int q = 0; q < 12; ++q) {
          if (a_is_I) acc.off(p, q) += off(p, q);
          else acc.off(q, p) += off(p, q);
        }
    }
    for (int k = 0; k < 144; ++k) dB.a[k] += hB.a[k];
    for (int p = 0; p < 12; ++p) grB[p] += gB[p];
  }
  if (a_dyn) {
    for (int k = 0; k < 144; ++k) dA.a[k] += hA.a[k];
    for (int p = 0; p < 12; ++p) grA[p] += gA[p];
  }
}

static inline const double* rest_of(const Scene& s, int body, int v) { return &s.rest[3 * (s.b[body].v_off + v)]; }

// ABD::ipc (abd.cpp:305-405) for one overlap's PT and EE pairs.
static void ipc_overlap(Scene& s, int o, OverlapAccum& acc) {
  const PairSet& P = s.set;
  int I = P.ov[o].I;
  for (int k = P.pt_off[o]; k < P.pt_off[o + 1]; ++k) {
    const I4& ij = P.pt[k];
    int A = ij[0], v = ij[1], B = ij[2], f = ij[3];
    V3 X[4];
    X[0] = Xat(s, A, v);
    face_at(s, s.X, B, f, X + 1);
    PTType ty = pt_type(X[0], X[1], X[2], X[3]);
    double d = pt_dist(X[0], X[1], X[2], X[3], ty);
    if (!(d < s.bp.dhat)) continue;
    // pt_uktk
    Mat<2, 12> TkT;
    pt_frame(X, ty, TkT);
    V3 X0[4];
    X0[0] = s.X0[s.b[A].v_off + v];
    face_at(s, s.X0, B, f, X0 + 1);
    double uk[2] = {0, 0};
    for (int i = 0; i < 4; ++i)
      for (int r = 0; r < 3; ++r) {
        double du = X[i][r] - X0[i][r];
        uk[0] += TkT(0, 3 * i + r) * du;
        uk[1] += TkT(1, 3 * i + r) * du;
      }
    double lam = -barrier_d1(d, s.bp) * 2 * std::sqrt(d);
    s.pt_tk[k] = TkT;
    s.pt_lam[k] = lam;
    M12 H;
    V12 g;
    ipc_hess_pt(X, ty, d, s.bp, s.cfg.psd != 0, H, g);
    if (s.cfg.pt_fric) friction<12>(uk, lam, transpose(TkT), g, H, s.fp);
    const double* xr[4];
    xr[0] = rest_of(s, A, v);
    const int* fc = &s.faces[3 * (s.b[B].f_off + f)];
    for (int i = 0; i < 3; ++i) xr[1 + i] = rest_of(s, B, fc[i]);
    chain_scatter(s, H, g, xr, 1, A, B, acc, A == I);
  }
  for (int k = P.ee_off[o]; k < P.ee_off[o + 1]; ++k) {
    const I4& ij = P.ee[k];
    int A = ij[0], ea = ij[1], B = ij[2], eb = ij[3];
    V3 X[4];
    edge_at(s, s.X, A, ea, X);
    edge_at(s, s.X, B, eb, X + 2);
    EEType ty = ee_type(X[0], X[1], X[2], X[3]);
    double d = ee_dist(X[0], X[1], X[2], X[3], ty);
    if (!(d < s.bp.dhat)) continue;
    M12 H;
    V12 g;
    ipc_hess_ee(X, ty, d, s.bp, s.cfg.eps_x, s.cfg.psd != 0, H, g);
    Mat<2, 12> TkT;
    ee_frame(X, ty, TkT);
    V3 X0[4];
    edge_at(s, s.X0, A, ea, X0);
    edge_at(s, s.X0, B, eb, X0 + 2);
    double uk[2] = {0, 0};
    for (int i = 0; i < 4; ++i)
      for (int r = 0; r < 3; ++r) {
        double du = X[i][r] - X0[i][r];
        uk[0] += TkT(0, 3 * i + r) * du;
        uk[1] += TkT(1, 3 * i + r) * du;
      }
    double lam = -barrier_d1(d, s.bp) * 2 * std::sqrt(d);
    s.ee_tk[k] = TkT;
    s.ee_lam[k] = lam;
    if (s.cfg.ee_fric) friction<12>(uk, lam, transpose(TkT), g, H, s.fp);
    const double* xr[4];
    const int* ed0 = &s.edges[2 * (s.b[A].e_off + ea)];
    const int* ed1 = &s.edges[2 * (s.b[B].e_off + eb)];
    xr[0] = rest_of(s, A, ed0[0]);
    xr[1] = rest_of(s, A, ed0[1]);
    xr[2] = rest_of(s, B, ed1[0]);
    xr[3] = rest_of(s, B, ed1[1]);
    chain_scatter(s, H, g, xr, 2, A, B, acc, A == I);
  }
}

// Block-sparse symmetric system: diagonal blocks + upper blocks (I < J).
struct BlockSys {
  int n;
  std::vector<M12> diag;
  std::map<std::pair<int, int>, M12> off;
  std::vector<double> rhs;  // gradient r (12 n)
};

// Per-body inertia terms + VG terms (abd.cpp:68-74, 380-401; vg_ipc.cpp:12-30).
static void body_terms(Scene& s) {
  int nb = (int)s.b.size();
  double dt = s.cfg.dt;
#pragma omp parallel for schedule(static)
  for (int I = 0; I < nb; ++I) {
    Body& c = s.b[I];
    if (c.mass < 0.0) {
      for (int i = 0; i < 12; ++i) c.grad[i] = 0;
      c.hess = M12();
      for (int i = 0; i < 12; ++i) c.hess(i, i) = 1.0;
      continue;
    }
    double og[12], qt[12];
    ortho_grad(c.q, s.cfg.ortho_kappa, og);
    q_tilde(s, c, qt);
    for (int i = 0; i < 12; ++i) {
      double m = i < 3 ? c.mass : c.Ic;
      c.grad[i] = dt * dt * og[i] + m * (c.q[i] - qt[i]);
    }
    M12 oh;
    ortho_hess(c.q, s.cfg.ortho_kappa, oh);
    for (int i = 0; i < 12; ++i)
      for (int j = 0; j < 12; ++j) c.hess(i, j) = (i == j ? (i < 3 ? c.mass : c.Ic) : 0.0) + oh(i, j) * dt * dt;
  }
  // VG (serial loop in the reference; contributions to each body summed in vertex order)
  int ng = (int)s.set.vg.size();
  s.g_lam.assign(ng, 0.0);
  for (int k = 0; k < ng; ++k) {
    int I = s.set.vg[k][0], v = s.set.vg[k][1];
    Body& c = s.b[I];
    V3 p = s.X[c.v_off + v];
    double _d = p.y + s.cfg.ground_offset;
    double d = _d * _d;
    if (!(d < s.bp.dhat)) continue;
    V3 p0 = s.X0[c.v_off + v];
    double uk[2] = {p.x - p0.x, p.z - p0.z};
    s.g_lam[k] = -barrier_d1(d, s.bp) * 2 * _d;
    if (c.mass < 0.0) continue;
    const double* xr = rest_of(s, I, v);
    double J[3][12];
    jac_rows(xr, J);
    // barrier_gradient_q, barrier_hessian_q (barrier.cpp:31-69)
    double b1 = barrier_d1(d, s.bp), b2 = barrier_d2(d, s.bp);
    double gy[12];
    for (int i = 0; i < 12; ++i) gy[i] = J[1][i];
    for (int i = 0; i < 12; ++i) c.grad[i] += gy[i] * (b1 * 2 * _d);
    for (int i = 0; i < 12; ++i)
      for (int j = 0; j < 12; ++j) c.hess(i, j) += b2 * (gy[i] * _d * 2) * (gy[j] * _d * 2);
    if (s.cfg.vg_fric) {
      Mat<12, 2> Tk;
      for (int i = 0; i < 12; ++i) {
        Tk(i, 0) = J[0][i];
        Tk(i, 1) = J[2][i];
      }
      Mat<12, 1> g;
      for (int i = 0; i < 12; ++i) g(i, 0) = c.grad[i];
      friction<12>(uk, s.g_lam[k], Tk, g, c.hess, s.fp);
      for (int i = 0; i < 12; ++i) c.grad[i] = g(i, 0);
    }
  }
}

// Assembles the Newton system of the current pair set at the current q
// (abd.cpp:68-89 + ipc()); positions: X at q, X0 at q0.
static void assemble(Scene& s, BlockSys& sys) {
  int nb = (int)s.b.size();
  project_all(s, 0);
  project_all(s, 1);
  body_terms(s);
  const PairSet& P = s.set;
  int nov = (int)P.ov.size();
  s.pt_tk.assign(P.pt.size(), Mat<2, 12>());
  s.ee_tk.assign(P.ee.size(), Mat<2, 12>());
  s.pt_lam.assign(P.pt.size(), 0.0);
  s.ee_lam.assign(P.ee.size(), 0.0);
  std::vector<OverlapAccum> acc(nov);
#pragma omp parallel for schedule(dynamic, 1)
  for (int o = 0; o < nov; ++o) {
    OverlapAccum& a = acc[o];
    a.off = M12(); a.dI = M12(); a.dJ = M12();
    for (int i = 0; i < 12; ++i) a.gI[i] = a.gJ[i] = 0;
    ipc_overlap(s, o, a);
  }
  sys.n = nb;
  sys.diag.assign(nb, M12());
  sys.off.clear();
  sys.rhs.assign(12 * nb, 0.0);
  for (int I = 0; I < nb; ++I) {
    for (int i = 0; i < 12; ++i) sys.rhs[12 * I + i] = s.b[I].grad[i];
  }
  for (int o = 0; o < nov; ++o) {
    int I = P.ov[o].I, J = P.ov[o].J;
    bool any = P.pt_off[o + 1] > P.pt_off[o] || P.ee_off[o + 1] > P.ee_off[o];
    if (!any) continue;
    for (int k = 0; k < 144; ++k) {
      sys.diag[I].a[k] += acc[o].dI.a[k];
      sys.diag[J].a[k] += acc[o].dJ.a[k];
    }
    for (int i = 0; i < 12; ++i) {
      sys.rhs[12 * I + i] += acc[o].gI[i];
      sys.rhs[12 * J + i] += acc[o].gJ[i];
    }
    sys.off[{I, J}] = acc[o].off;
  }
  for (int I = 0; I < nb; ++I)
    for (int k = 0; k < 144; ++k) sys.diag[I].a[k] += s.b[I].hess.a[k];
  if (s.cfg.damp) {
    // damping_sparse (mutils.cpp:106-115): every entry scaled by 1 + beta, then
    // mass (translation) or Ic (the rest) times alpha - beta on the diagonal
    double sc = 1 + s.cfg.damp_beta, dab = s.cfg.damp_alpha - s.cfg.damp_beta;
    for (int I = 0; I < nb; ++I) {
      for (int k = 0; k < 144; ++k) sys.diag[I].a[k] *= sc;
      for (int j = 0; j < 12; ++j) sys.diag[I].a[13 * j] += (j < 3 ? s.b[I].mass : s.b[I].Ic) * dab;
    }
    for (auto& kv : sys.off)
      for (int k = 0; k < 144; ++k) kv.second.a[k] *= sc;
  }
}

// ---------------------------------------------------------------------------------
// Direct block-sparse Cholesky with a greedy minimum-degree ordering (stands in for
// PardisoLLT, abd.cpp:270-272). Returns false if the matrix is not positive definite.
static bool chol12(M12& A) {
  for (int j = 0; j < 12; ++j) {
    double s = A(j, j);
    for (int k = 0; k < j; ++k) s -= A(j, k) * A(j, k);
    if (!(s > 0)) return false;
    double l = std::sqrt(s);
    A(j, j) = l;
    for (int i = j + 1; i < 12; ++i) {
      double t = A(i, j);
      for (int k = 0; k < j; ++k) t -= A(i, k) * A(j, k);
      A(i, j) = t / l;
    }
    for (int i = 0; i < j; ++i) A(i, j) = 0;
  }
  return true;
}

static bool block_cholesky_solve(const BlockSys& sys, std::vector<double>& x) {
  int n = sys.n;
  std::vector<std::set<int>> adj(n);
  for (auto& kv : sys.off) {
    adj[kv.first.first].insert(kv.first.second);
    adj[kv.first.second].insert(kv.first.first);
  }
  // greedy minimum degree
  std::vector<int> perm, inv(n, -1);
  std::vector<std::vector<int>> strct(n);  // later-eliminated neighbours at elimination
  {
    std::vector<std::set<int>> g = adj;
    std::set<std::pair<int, int>> pq;
    for (int i = 0; i < n; ++i) pq.insert({(int)g[i].size(), i});
    while (!pq.empty()) {
      int v = pq.begin()->second;
      pq.erase(pq.begin());
      inv[v] = (int)perm.size();
      perm.push_back(v);
      std::vector<int> nb(g[v].begin(), g[v].end());
      strct[v] = nb;
      for (int a : nb) {
        pq.erase({(int)g[a].size(), a});
        g[a].erase(v);
      }
      for (size_t i = 0; i < nb.size(); ++i)
        for (size_t j = i + 1; j < nb.size(); ++j) {
          g[nb[i]].insert(nb[j]);
          g[nb[j]].insert(nb[i]);
        }
      for (int a : nb) pq.insert({(int)g[a].size(), a});
    }
  }
  // storage: L blocks keyed (row, col) in original ids, row eliminated after col
  std::vector<M12> D(n);
  for (int i = 0; i < n; ++i) D[i] = sys.diag[i];
  std::vector<std::unordered_map<int, M12>> Lc(n);  // column v -> {row -> block}
  for (int v = 0; v < n; ++v)
    for (int r : strct[v]) Lc[v][r] = M12();
  for (auto& kv : sys.off) {
    int a = kv.first.first, b = kv.first.second;  // block (a, b)
    if (inv[a] > inv[b]) Lc[b][a] = kv.second;     // row a, col b
    else Lc[a][b] = transpose(kv.second);          // row b, col a = (a,b)^T
  }
  for (int k = 0; k < n; ++k) {
    int v = perm[k];
    if (!chol12(D[v])) return false;
    // L_rv = A_rv L_vv^{-T}
    std::vector<int> rows = strct[v];
    std::sort(rows.begin(), rows.end(), [&](int a, int b) { return inv[a] < inv[b]; });
    for (int r : rows) {
      M12& B = Lc[v][r];
      // solve X L^T = B for X (row by row: forward on L)
      for (int i = 0; i < 12; ++i)
        for (int j = 0; j < 12; ++j) {
          double t = B(i, j);
          for (int m = 0; m < j; ++m) t -= B(i, m) * D[v](j, m);
          B(i, j) = t / D[v](j, j);
        }
    }
    int nr = (int)rows.size();
    // Schur updates A_ab -= L_av L_bv^T for a, b in rows (a eliminated after/equal b)
#pragma omp parallel for schedule(dynamic, 1) if (nr > 8)
    for (int ia = 0; ia < nr; ++ia) {
      int a = rows[ia];
      const M12& La = Lc[v].at(a);
      for (int ib = 0; ib <= ia; ++ib) {
        int bb = rows[ib];
        const M12& Lb = Lc[v].at(bb);
        M12 U;
        for (int i = 0; i < 12; ++i)
          for (int j = 0; j < 12; ++j) {
            double t = 0;
            for (int m = 0; m < 12; ++m) t += La(i, m) * Lb(j, m);
            U(i, j) = t;
          }
        if (a == bb) {
          for (int q = 0; q < 144; ++q) D[a].a[q] -= U.a[q];
        } else {
          // block (a, bb) with a after bb: stored in column bb, row a
          M12& T = Lc[bb].at(a);
          for (int q = 0; q < 144; ++q) T.a[q] -= U.a[q];
        }
      }
    }
  }
  // forward: L y = b (in elimination order)
  std::vector<double> y(sys.rhs);
  for (int k = 0; k < n; ++k) {
    int v = perm[k];
    double* yv = &y[12 * v];
    for (int i = 0; i < 12; ++i) {
      double t = yv[i];
      for (int m = 0; m < i; ++m) t -= D[v](i, m) * yv[m];
      yv[i] = t / D[v](i, i);
    }
    for (auto& kv : Lc[v]) {
      double* yr = &y[12 * kv.first];
      for (int i = 0; i < 12; ++i) {
        double t = 0;
        for (int m = 0; m < 12; ++m) t += kv.second(i, m) * yv[m];
        yr[i] -= t;
      }
    }
  }
  // backward: L^T x = y
  for (int k = n - 1; k >= 0; --k) {
    int v = perm[k];
    double* yv = &y[12 * v];
    for (auto& kv : Lc[v]) {
      const double* xr = &y[12 * kv.first];
      for (int m = 0; m < 12; ++m) {
        double t = 0;
        for (int i = 0; i < 12; ++i) t += kv.second(i, m) * xr[i];
        yv[m] -= t;
      }
    }
    for (int i = 11; i >= 0; --i) {
      double t = yv[i];
      for (int m = i + 1; m < 12; ++m) t -= D[v](m, i) * yv[m];
      yv[i] = t / D[v](i, i);
    }
  }
  x = y;
  return true;
}

// ---------------------------------------------------------------------------------
// Energies of the line search (energy.cpp:19-86, 195-270), one function per term so the
// totals and the per-pair values of orc_energy_terms come from the same arithmetic.
// Positions are those of the last project_all (s.X at q + dq, s.X0 at q0).
static double pt_barrier_energy(Scene& s, const I4& ij) {  // energy.cpp:34-50
  V3 X[4];
  X[0] = Xat(s, ij[0], ij[1]);
  face_at(s, s.X, ij[2], ij[3], X + 1);
  PTType t = pt_type(X[0], X[1], X[2], X[3]);
  return barrier(pt_dist(X[0], X[1], X[2], X[3], t), s.bp);
}
static double ee_barrier_energy(Scene& s, const I4& ij) {  // energy.cpp:52-80, mollified
  V3 X[4];
  edge_at(s, s.X, ij[0], ij[1], X);
  edge_at(s, s.X, ij[2], ij[3], X + 2);
  double eps_x = sqnorm(X[0] - X[1]) * sqnorm(X[2] - X[3]) * s.cfg.eps_x;
  double m;
  V3 u = X[1] - X[0], v = X[3] - X[2];
  double x = sqnorm(cross(u, v));
  if (x < eps_x) {
    double xe = x / eps_x;
    m = (-xe + 2.0) * xe;
  } else {
    m = 1.0;
  }
  EEType t = ee_type(X[0], X[1], X[2], X[3]);
  return barrier(ee_dist(X[0], X[1], X[2], X[3], t), s.bp) * m;
}
static double vg_barrier_energy(Scene& s, const std::array<int, 2>& iv) {  // E_ground, energy.cpp:261-270
  V3 p = Xat(s, iv[0], iv[1]);
  double d = p.y + s.cfg.ground_offset;
  d = d * d;
  return d < s.bp.dhat ? barrier(d, s.bp) : 0.0;
}
// Lagged friction of pair k of the current set (E_fric, energy.cpp:195-258): tangent
// displacement Tk (x - x0) of the pair's four vertices.
static double pair_friction_energy(Scene& s, int kind, int k) {
  const I4& ij = kind ? s.set.ee[k] : s.set.pt[k];
  V3 X[4], X0[4];
  if (kind) {
    edge_at(s, s.X, ij[0], ij[1], X);
    edge_at(s, s.X, ij[2], ij[3], X + 2);
    edge_at(s, s.X0, ij[0], ij[1], X0);
    edge_at(s, s.X0, ij[2], ij[3], X0 + 2);
  } else {
    X[0] = Xat(s, ij[0], ij[1]);
    face_at(s, s.X, ij[2], ij[3], X + 1);
    X0[0] = s.X0[s.b[ij[0]].v_off + ij[1]];
    face_at(s, s.X0, ij[2], ij[3], X0 + 1);
  }
  const auto& Tk = kind ? s.ee_tk[k] : s.pt_tk[k];
  double u0 = 0, u1 = 0;
  for (int i = 0; i < 4; ++i)
    for (int r = 0; r < 3; ++r) {
      double du = X[i][r] - X0[i][r];
      u0 += Tk(0, 3 * i + r) * du;
      u1 += Tk(1, 3 * i + r) * du;
    }
  double lam = kind ? s.ee_lam[k] : s.pt_lam[k];
  return s.fp.mu * lam * f0_SF(std::sqrt(u0 * u0 + u1 * u1), s.fp.epsv);
}
static double vg_friction_energy(Scene& s, int k) {  // ground friction in the x, z plane
  int I = s.set.vg[k][0], v = s.set.vg[k][1];
  V3 d = s.X[s.b[I].v_off + v] - s.X0[s.b[I].v_off + v];
  return s.fp.mu * s.g_lam[k] * f0_SF(std::sqrt(d.x * d.x + d.z * d.z), s.fp.epsv);
}

// Inertia + orthogonality of every body at q + dqk (the bodies' dq is set to dqk).
static double E_inert(Scene& s, const std::vector<double>& dqk) {
  int nb = (int)s.b.size();
  double e = 0;
  for (int I = 0; I < nb; ++I) {
    Body& c = s.b[I];
    for (int i = 0; i < 12; ++i) c.dq[i] = dqk[12 * I + i];
    double q1[12];
    q_plus(c.q, c.dq, q1);
    e += inertia_energy(s, c, q1);
  }
  return e;
}

static double E_barrier_plus_inert(Scene& s, const PairSet& P, const std::vector<double>& dqk) {
  double e = E_inert(s, dqk);
  project_all(s, 2);
  double ep = 0, ee_ = 0, eg = 0;
  if (s.cfg.pt) {
#pragma omp parallel for reduction(+ : ep) schedule(static)
    for (int k = 0; k < (int)P.pt.size(); ++k) ep += pt_barrier_energy(s, P.pt[k]);
  }
  if (s.cfg.ee) {
#pragma omp parallel for reduction(+ : ee_) schedule(static)
    for (int k = 0; k < (int)P.ee.size(); ++k) ee_ += ee_barrier_energy(s, P.ee[k]);
  }
  if (s.cfg.ground) {
    for (int k = 0; k < (int)P.vg.size(); ++k) eg += vg_barrier_energy(s, P.vg[k]);
  }
  return e + ep + ee_ + eg;
}

static double E_fric(Scene& s, const std::vector<double>& dqk) {
  int nb = (int)s.b.size();
  for (int I = 0; I < nb; ++I)
    for (int i = 0; i < 12; ++i) s.b[I].dq[i] = dqk[12 * I + i];
  project_all(s, 2);
  const PairSet& P = s.set;
  double ef = 0;
  if (s.cfg.pt && s.cfg.pt_fric) {
#pragma omp parallel for reduction(+ : ef) schedule(static)
    for (int k = 0; k < (int)P.pt.size(); ++k) ef += pair_friction_energy(s, 0, k);
  }
  if (s.cfg.ee && s.cfg.ee_fric) {
#pragma omp parallel for reduction(+ : ef) schedule(static)
    for (int k = 0; k < (int)P.ee.size(); ++k) ef += pair_friction_energy(s, 1, k);
  }
  if (s.cfg.ground && s.cfg.vg_fric) {
    for (int k = 0; k < (int)P.vg.size(); ++k) ef += vg_friction_energy(s, k);
  }
  return ef;
}

// ABD::line_search (line_search.cpp:39-136). Returns the accepted alpha and adopts the
// pair set culled at q + alpha dq.
static double line_search(Scene& s, const std::vector<double>& dq, const std::vector<double>& r, int& trials) {
  int n = (int)dq.size();
  double alpha = 1.0;
  std::vector<double> zero(n, 0.0);
  double E0 = E_barrier_plus_inert(s, s.set, zero) + E_fric(s, zero);
  double qdg = 0, gn = 0, dqn = 0;
  for (int i = 0; i < n; ++i) {
    qdg += dq[i] * r[i];
    gn += r[i] * r[i];
    dqn += dq[i] * dq[i];
  }
  gn = std::sqrt(gn);
  dqn = std::sqrt(dqn);
  PairSet Pn;
  std::vector<double> dqk(n);
  trials = 0;
  for (int guard = 0; guard < 2200; ++guard) {
    for (int i = 0; i < n; ++i) dqk[i] = dq[i] * alpha;
    for (int I = 0; I < (int)s.b.size(); ++I)
      for (int i = 0; i < 12; ++i) s.b[I].dq[i] = dqk[12 * I + i];
    cull(s, 2, &Pn);
    double E3 = E_barrier_plus_inert(s, Pn, dqk);
    double ef = E_fric(s, dqk);
    double E1 = E3 + ef;
    ++trials;
    bool wolfe = E1 <= E0 + s.cfg.c1 * alpha * qdg;
    alpha /= 2;
    if (!(!wolfe && gn > s.cfg.ls_grad_tol)) break;
    if (dqn * alpha * 2 < s.cfg.tol && s.cfg.clip) {
      alpha = 0.0;
      break;
    }
  }
  s.set = Pn;
  return alpha * 2;
}

// ---------------------------------------------------------------------------------
static double now_s() { return omp_get_wtime(); }

// ABD::implicit_euler (abd.cpp:30-140).
static int implicit_euler(Scene& s) {
  int nb = (int)s.b.size();
  double dt = s.cfg.dt;
  Stats& st = s.st;
  st = Stats{};
  st.toi_min = 1.0;
  st.alpha_min = 1.0;
  for (auto& c : s.b) std::memcpy(c.q, c.q0, sizeof(c.q));
  for (auto& c : s.b) std::memset(c.dq, 0, sizeof(c.dq));
  cull(s, 1, &s.set);
  bool term;
  do {
    double t0 = now_s();
    BlockSys sys;
    assemble(s, sys);
    st.n_pt = std::max(st.n_pt, (int)s.set.pt.size());
    st.n_ee = std::max(st.n_ee, (int)s.set.ee.size());
    st.n_vg = std::max(st.n_vg, (int)s.set.vg.size());
    double t1 = now_s();
    std::vector<double> x;
    if (!block_cholesky_solve(sys, x)) return st.status = ST_NOT_SPD;
    std::vector<double> dq(12 * nb);
    double nrm = 0;
    for (int i = 0; i < 12 * nb; ++i) {
      dq[i] = -x[i];
      nrm += dq[i] * dq[i];
    }
    if (std::isnan(std::sqrt(nrm))) return st.status = ST_NAN;
    double t2 = now_s();
    // ccd (abd.cpp:142-196)
    double toi = 1.0, factor = 1.0;
    double sup_dq = std::sqrt(nrm);
    for (int I = 0; I < nb; ++I)
      for (int i = 0; i < 12; ++i) s.b[I].dq[i] = dq[12 * I + i];
    if (s.cfg.upper_bound) toi = cull(s, 3, nullptr);
    if ((s.cfg.ground && s.g_cnt > 1) || s.p_cnt > 1) return st.status = ST_TOI_TINY;
    if (toi < 1.0) factor = s.cfg.backoff;
    st.toi_min = std::min(st.toi_min, toi);
    // same-direction stop (abd.cpp:180-190); with dq_tol = 0 it can never trigger
    if (s.iter && s.lastdq.size() == dq.size()) {
      double dl = 0, ll = 0, df = 0;
      for (int i = 0; i < 12 * nb; ++i) {
        dl += dq[i] * s.lastdq[i];
        ll += s.lastdq[i] * s.lastdq[i];
        df += (dq[i] - s.lastdq[i]) * (dq[i] - s.lastdq[i]);
      }
      double c = dl / (std::sqrt(nrm) * std::sqrt(ll));
      if (std::fabs(c) > 1.0 - s.cfg.dq_tol && std::sqrt(df) / std::sqrt(nrm) < s.cfg.dq_tol)
        return st.status = ST_SAME_DIR;
    }
    s.lastdq = dq;
    for (auto& v : dq) v *= factor * toi;
    double t3 = now_s();
    // line search (abd.cpp:198-227)
    double alpha = 1.0;
    int trials = 0;
    if (s.cfg.line_search) alpha = line_search(s, dq, sys.rhs, trials);
    st.ls_trials += trials;
    st.alpha_min = std::min(st.alpha_min, alpha);
    for (auto& v : dq) v *= alpha;
    for (int I = 0; I < nb; ++I)
      for (int i = 0; i < 12; ++i) s.b[I].q[i] += dq[12 * I + i];
    double t4 = now_s();
    st.t_ipc += t1 - t0;
    st.t_solver += t2 - t1;
    st.t_ccd += t3 - t2;
    st.t_ls += t4 - t3;
    st.newton_iters++;
    term = sup_dq < s.cfg.tol || ++s.iter >= s.cfg.max_iter;
    if (s.cfg.max_iter_frame > 0 && st.newton_iters >= s.cfg.max_iter_frame) term = true;
  } while (!term);
  ++s.iter;  // abd.cpp:121 increments the counter once more per frame
  for (auto& c : s.b) {
    for (int i = 0; i < 12; ++i) {
      c.dqdt[i] = (c.q[i] - c.q0[i]) / dt;
      c.q0[i] = c.q[i];
    }
  }
  return st.status = ST_OK;
}

}  // namespace orc

using namespace orc;

// ---------------------------------------------------------------------------------
// C API used by tests and bench.py (ctypes). Config layout mirrors struct Config.
extern "C" {

void* orc_create(int nb, const double* q0, const double* dqdt, const double* mass, const double* Ic,
                 const int* vert_off, const double* rest, const int* edge_off, const int* edges,
                 const int* face_off, const int* faces, const Config* cfg) {
  Scene* s = new Scene();
  s->cfg = *cfg;
  s->bp = BarrierParams{cfg->dhat, cfg->kappa};
  s->fp = FrictionParams{cfg->mu, cfg->dt * cfg->evh, cfg->max_uk};
  s->d_sqrt = std::sqrt(cfg->dhat);
  if (cfg->n_threads > 0) omp_set_num_threads(cfg->n_threads);
  s->b.resize(nb);
  int nv = vert_off[nb], ne = edge_off[nb], nf = face_off[nb];
  s->rest.assign(rest, rest + 3 * nv);
  s->edges.assign(edges, edges + 2 * ne);
  s->faces.assign(faces, faces + 3 * nf);
  s->X.resize(nv);
  s->Xq.resize(nv);
  s->X0.resize(nv);
  s->nv_tot = nv;
  for (int I = 0; I < nb; ++I) {
    Body& c = s->b[I];
    std::memcpy(c.q0, q0 + 12 * I, sizeof(c.q0));
    std::memcpy(c.q, q0 + 12 * I, sizeof(c.q));
    std::memcpy(c.dqdt, dqdt + 12 * I, sizeof(c.dqdt));
    std::memset(c.dq, 0, sizeof(c.dq));
    c.mass = mass[I];
    c.Ic = Ic[I];
    c.v_off = vert_off[I];
    c.nv = vert_off[I + 1] - vert_off[I];
    c.e_off = edge_off[I];
    c.ne = edge_off[I + 1] - edge_off[I];
    c.f_off = face_off[I];
    c.nf = face_off[I + 1] - face_off[I];
    V3 lo, hi;
    for (int v = 0; v < c.nv; ++v) {
      const double* p = &s->rest[3 * (c.v_off + v)];
      V3 pv(p[0], p[1], p[2]);
      if (v == 0) lo = hi = pv;
      else { lo = vmin(lo, pv); hi = vmax(hi, pv); }
    }
    c.rest = inflate(Box{lo, hi}, s->d_sqrt);
  }
  return s;
}

void orc_destroy(void* h) { delete (Scene*)h; }

int orc_step(void* h, int n_frames, Stats* stats) {
  Scene& s = *(Scene*)h;
  Stats acc{};
  acc.toi_min = 1.0;
  acc.alpha_min = 1.0;
  int rc = 0;
  for (int f = 0; f < n_frames; ++f) {
    rc = implicit_euler(s);
    acc.newton_iters += s.st.newton_iters;
    acc.ls_trials += s.st.ls_trials;
    acc.n_pt = std::max(acc.n_pt, s.st.n_pt);
    acc.n_ee = std::max(acc.n_ee, s.st.n_ee);
    acc.n_vg = std::max(acc.n_vg, s.st.n_vg);
    acc.toi_min = std::min(acc.toi_min, s.st.toi_min);
    acc.alpha_min = std::min(acc.alpha_min, s.st.alpha_min);
    acc.t_ipc += s.st.t_ipc;
    acc.t_solver += s.st.t_solver;
    acc.t_ccd += s.st.t_ccd;
    acc.t_ls += s.st.t_ls;
    if (rc) break;
  }
  acc.status = rc;
  if (stats) *stats = acc;
  return rc;
}

void orc_get_state(void* h, double* q0, double* dqdt) {
  Scene& s = *(Scene*)h;
  for (size_t I = 0; I < s.b.size(); ++I) {
    if (q0) std::memcpy(q0 + 12 * I, s.b[I].q0, 12 * sizeof(double));
    if (dqdt) std::memcpy(dqdt + 12 * I, s.b[I].dqdt, 12 * sizeof(double));
  }
}
void orc_set_state(void* h, const double* q0, const double* dqdt) {
  Scene& s = *(Scene*)h;
  for (size_t I = 0; I < s.b.size(); ++I) {
    if (q0) { std::memcpy(s.b[I].q0, q0 + 12 * I, 12 * sizeof(double)); std::memcpy(s.b[I].q, q0 + 12 * I, 12 * sizeof(double)); }
    if (dqdt) std::memcpy(s.b[I].dqdt, dqdt + 12 * I, 12 * sizeof(double));
  }
}
int orc_get_iter(void* h) { return ((Scene*)h)->iter; }
void orc_set_iter(void* h, int it) { ((Scene*)h)->iter = it; }

// Culling at an explicit state: q (12 nb) and dq (12 nb, may be null). vtn 1/2 store
// the pair set (read back with orc_get_pairs); vtn 3 returns the TOI.
double orc_cull(void* h, int vtn, const double* q, const double* dq, int* counts) {
  Scene& s = *(Scene*)h;
  for (size_t I = 0; I < s.b.size(); ++I) {
    std::memcpy(s.b[I].q, q + 12 * I, 12 * sizeof(double));
    if (dq) std::memcpy(s.b[I].dq, dq + 12 * I, 12 * sizeof(double));
    else std::memset(s.b[I].dq, 0, 12 * sizeof(double));
  }
  double t = cull(s, vtn, vtn == 3 ? nullptr : &s.set);
  if (counts) {
    counts[0] = (int)s.set.pt.size();
    counts[1] = (int)s.set.ee.size();
    counts[2] = (int)s.set.vg.size();
    counts[3] = (int)s.set.ov.size();
  }
  return t;
}
void orc_get_pairs(void* h, int* pt, int* pt_ty, int* ee, int* ee_ty, int* vg) {
  Scene& s = *(Scene*)h;
  for (size_t k = 0; k < s.set.pt.size(); ++k) {
    for (int i = 0; i < 4; ++i) pt[4 * k + i] = s.set.pt[k][i];
    pt_ty[k] = s.set.pt_ty[k];
  }
  for (size_t k = 0; k < s.set.ee.size(); ++k) {
    for (int i = 0; i < 4; ++i) ee[4 * k + i] = s.set.ee[k][i];
    ee_ty[k] = s.set.ee_ty[k];
  }
  for (size_t k = 0; k < s.set.vg.size(); ++k) {
    vg[2 * k] = s.set.vg[k][0];
    vg[2 * k + 1] = s.set.vg[k][1];
  }
}

// Newton system at state (q, current q0/dqdt) for the pair set culled at q.
// Outputs: grad (12 nb), diag (144 nb row-major), n_off blocks with keys (I<J) and
// values (144 each, block (I, J) row-major). Returns the number of off blocks; when
// off_keys is null only the count is returned.
int orc_newton_system(void* h, const double* q, double* grad, double* diag, int* off_keys, double* off_vals,
                      int max_off) {
  Scene& s = *(Scene*)h;
  for (size_t I = 0; I < s.b.size(); ++I) {
    std::memcpy(s.b[I].q, q + 12 * I, 12 * sizeof(double));
    std::memset(s.b[I].dq, 0, 12 * sizeof(double));
  }
  cull(s, 1, &s.set);
  BlockSys sys;
  assemble(s, sys);
  int nb = (int)s.b.size();
  if (grad) std::memcpy(grad, sys.rhs.data(), 12 * nb * sizeof(double));
  if (diag)
    for (int I = 0; I < nb; ++I) std::memcpy(diag + 144 * I, sys.diag[I].a, 144 * sizeof(double));
  int k = 0;
  if (off_keys) {
    for (auto& kv : sys.off) {
      if (k >= max_off) break;
      off_keys[2 * k] = kv.first.first;
      off_keys[2 * k + 1] = kv.first.second;
      std::memcpy(off_vals + 144 * k, kv.second.a, 144 * sizeof(double));
      ++k;
    }
    return k;
  }
  return (int)sys.off.size();
}

// Solves the Newton system at q with the direct solver: dq = -H^{-1} r.
int orc_newton_dq(void* h, const double* q, double* dq) {
  Scene& s = *(Scene*)h;
  for (size_t I = 0; I < s.b.size(); ++I) {
    std::memcpy(s.b[I].q, q + 12 * I, 12 * sizeof(double));
    std::memset(s.b[I].dq, 0, 12 * sizeof(double));
  }
  cull(s, 1, &s.set);
  BlockSys sys;
  assemble(s, sys);
  std::vector<double> x;
  if (!block_cholesky_solve(sys, x)) return ST_NOT_SPD;
  for (size_t i = 0; i < x.size(); ++i) dq[i] = -x[i];
  return 0;
}

// Line-search energy terms at q + dq with the friction lagged at q (the first trial of
// ABD::line_search at alpha = 1, line_search.cpp:88-110): culls at q, assembles there
// (lagged Tk, lambda), culls at q + dq, then evaluates.
// terms: [inertia + orthogonality, PT barrier, EE barrier, ground barrier, friction];
// counts: pairs of the set at q + dq (pt, ee, vg), then of the lagged set (pt, ee, vg);
// per-pair arrays (any may be null): barrier energies over the set at q + dq, friction
// energies over the lagged set (0 where the term is switched off).
int orc_energy_terms(void* h, const double* q, const double* dq, double* terms, int* counts, double* e_pt,
                     double* e_ee, double* e_vg, double* f_pt, double* f_ee, double* f_vg) {
  Scene& s = *(Scene*)h;
  int nb = (int)s.b.size();
  for (int I = 0; I < nb; ++I) {
    std::memcpy(s.b[I].q, q + 12 * I, 12 * sizeof(double));
    std::memset(s.b[I].dq, 0, 12 * sizeof(double));
  }
  cull(s, 1, &s.set);
  BlockSys sys;
  assemble(s, sys);
  std::vector<double> dqk(dq, dq + 12 * nb);
  for (int I = 0; I < nb; ++I) std::memcpy(s.b[I].dq, dq + 12 * I, 12 * sizeof(double));
  PairSet Pn;
  cull(s, 2, &Pn);
  double t[5] = {E_inert(s, dqk), 0, 0, 0, 0};
  project_all(s, 2);
  for (int k = 0; k < (int)Pn.pt.size(); ++k) {
    double e = s.cfg.pt ? pt_barrier_energy(s, Pn.pt[k]) : 0.0;
    if (e_pt) e_pt[k] = e;
    t[1] += e;
  }
  for (int k = 0; k < (int)Pn.ee.size(); ++k) {
    double e = s.cfg.ee ? ee_barrier_energy(s, Pn.ee[k]) : 0.0;
    if (e_ee) e_ee[k] = e;
    t[2] += e;
  }
  for (int k = 0; k < (int)Pn.vg.size(); ++k) {
    double e = s.cfg.ground ? vg_barrier_energy(s, Pn.vg[k]) : 0.0;
    if (e_vg) e_vg[k] = e;
    t[3] += e;
  }
  const PairSet& L = s.set;
  for (int k = 0; k < (int)L.pt.size(); ++k) {
    double e = (s.cfg.pt && s.cfg.pt_fric) ? pair_friction_energy(s, 0, k) : 0.0;
    if (f_pt) f_pt[k] = e;
    t[4] += e;
  }
  for (int k = 0; k < (int)L.ee.size(); ++k) {
    double e = (s.cfg.ee && s.cfg.ee_fric) ? pair_friction_energy(s, 1, k) : 0.0;
    if (f_ee) f_ee[k] = e;
    t[4] += e;
  }
  for (int k = 0; k < (int)L.vg.size(); ++k) {
    double e = (s.cfg.ground && s.cfg.vg_fric) ? vg_friction_energy(s, k) : 0.0;
    if (f_vg) f_vg[k] = e;
    t[4] += e;
  }
  if (terms)
    for (int i = 0; i < 5; ++i) terms[i] = t[i];
  if (counts) {
    counts[0] = (int)Pn.pt.size();
    counts[1] = (int)Pn.ee.size();
    counts[2] = (int)Pn.vg.size();
    counts[3] = (int)L.pt.size();
    counts[4] = (int)L.ee.size();
    counts[5] = (int)L.vg.size();
  }
  return 0;
}

// Scalar energy at q (inertia + barrier on the set culled at q; no friction).
double orc_energy(void* h, const double* q) {
  Scene& s = *(Scene*)h;
  for (size_t I = 0; I < s.b.size(); ++I) {
    std::memcpy(s.b[I].q, q + 12 * I, 12 * sizeof(double));
    std::memset(s.b[I].dq, 0, 12 * sizeof(double));
  }
  cull(s, 1, &s.set);
  std::vector<double> zero(12 * s.b.size(), 0.0);
  return E_barrier_plus_inert(s, s.set, zero);
}

void orc_stats_last(void* h, Stats* st) { *st = ((Scene*)h)->st; }

// ----- per-primitive functions (abdtk mirror and golden checks) -----
int orc_pt_type(const double* x) {
  V3 p(x[0], x[1], x[2]), a(x[3], x[4], x[5]), b(x[6], x[7], x[8]), c(x[9], x[10], x[11]);
  return pt_type(p, a, b, c);
}
double orc_pt_dist(const double* x, int ty) {
  V3 p(x[0], x[1], x[2]), a(x[3], x[4], x[5]), b(x[6], x[7], x[8]), c(x[9], x[10], x[11]);
  return pt_dist(p, a, b, c, (PTType)ty);
}
int orc_ee_type(const double* x) {
  V3 p(x[0], x[1], x[2]), a(x[3], x[4], x[5]), b(x[6], x[7], x[8]), c(x[9], x[10], x[11]);
  return ee_type(p, a, b, c);
}
double orc_ee_dist(const double* x, int ty) {
  V3 p(x[0], x[1], x[2]), a(x[3], x[4], x[5]), b(x[6], x[7], x[8]), c(x[9], x[10], x[11]);
  return ee_dist(p, a, b, c, (EEType)ty);
}
static void load4(const double* x, V3 X[4]) {
  for (int i = 0; i < 4; ++i) X[i] = V3(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
}
// ipc_hess_pt_12x12 (core_ipc.cpp:21-46): H row-major 144, g 12.
void orc_ipc_hess_pt(const double* x, int ty, double d, double dhat, double kappa, int psd, double* H, double* g) {
  V3 X[4];
  load4(x, X);
  M12 Hm;
  V12 gm;
  ipc_hess_pt(X, (PTType)ty, d, BarrierParams{dhat, kappa}, psd != 0, Hm, gm);
  std::memcpy(H, Hm.a, sizeof(Hm.a));
  std::memcpy(g, gm.a, sizeof(gm.a));
}
double orc_ipc_hess_ee(const double* x, int ty, double d, double dhat, double kappa, double eps_x, int psd,
                       double* H, double* g) {
  V3 X[4];
  load4(x, X);
  M12 Hm;
  V12 gm;
  double m = ipc_hess_ee(X, (EEType)ty, d, BarrierParams{dhat, kappa}, eps_x, psd != 0, Hm, gm);
  std::memcpy(H, Hm.a, sizeof(Hm.a));
  std::memcpy(g, gm.a, sizeof(gm.a));
  return m;
}
double orc_barrier(double d, double dhat, double kappa, int which) {
  BarrierParams bp{dhat, kappa};
  return which == 0 ? barrier(d, bp) : (which == 1 ? barrier_d1(d, bp) : barrier_d2(d, bp));
}
// pt_collision_time(p0_t0, t0_t0, t1_t0, t2_t0, p0_t1, ...) (collision.cpp:299-323)
double orc_pt_collision_time(const double* x) {
  V3 a[4], b[4];
  load4(x, a);
  load4(x + 12, b);
  return pt_collision_time(a[0], a + 1, b[0], b + 1);
}
// ee_collision_time(ei0_t0, ei1_t0, ej0_t0, ej1_t0, ei0_t1, ...) (collision.cpp:325-348)
double orc_ee_collision_time(const double* x) {
  V3 a[4], b[4];
  load4(x, a);
  load4(x + 12, b);
  V3 ei0[2] = {a[0], a[1]}, ej0[2] = {a[2], a[3]}, ei1[2] = {b[0], b[1]}, ej1[2] = {b[2], b[3]};
  return ee_collision_time(ei0, ej0, ei1, ej1);
}
int orc_cubic_roots(const double* c, double x0, double x1, double* roots) {
  return cubic_roots(roots, c, x0, x1);
}
// det_polynomial(a, b) with a, b row-major 3x3
void orc_det_polynomial(const double* a, const double* b, double* out) {
  M3c A, B;
  for (int r = 0; r < 3; ++r)
    for (int k = 0; k < 3; ++k) {
      A.col[k][r] = a[3 * r + k];
      B.col[k][r] = b[3 * r + k];
    }
  det_polynomial(A, B, out);
}
// Friction (friction.cpp:15-47) on a 12x2 Tk (row-major 24); adds into g, H.
void orc_friction(const double* uk, double lam, const double* Tk, double mu, double epsv, double max_uk, double* g,
                  double* H) {
  Mat<12, 2> T;
  std::memcpy(T.a, Tk, sizeof(T.a));
  Mat<12, 1> gg;
  std::memcpy(gg.a, g, sizeof(gg.a));
  M12 HH;
  std::memcpy(HH.a, H, sizeof(HH.a));
  friction<12>(uk, lam, T, gg, HH, FrictionParams{mu, epsv, max_uk});
  std::memcpy(g, gg.a, sizeof(gg.a));
  std::memcpy(H, HH.a, sizeof(HH.a));
}
double orc_f0(double x, double epsv) { return f0_SF(x, epsv); }
void orc_pt_frame(const double* x, int ty, double* TkT) {
  V3 X[4];
  load4(x, X);
  Mat<2, 12> T;
  pt_frame(X, (PTType)ty, T);
  std::memcpy(TkT, T.a, sizeof(T.a));
}
void orc_ee_frame(const double* x, int ty, double* TkT) {
  V3 X[4];
  load4(x, X);
  Mat<2, 12> T;
  ee_frame(X, (EEType)ty, T);
  std::memcpy(TkT, T.a, sizeof(T.a));
}
int orc_sizeof_config() { return (int)sizeof(Config); }
int orc_sizeof_stats() { return (int)sizeof(Stats); }

}  // extern "C"
