// Internal declarations shared by the CUDA translation units of libabd_gb300.so:
// device buffers, the pair-set layout in HBM, and the host-side launchers of each stage.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/abd_gb300.h"

namespace abd {

struct CudaError {
  cudaError_t code;
  std::string where;
};
void check(cudaError_t e, const char* where);  // throws CudaError
#define CK(x) ::abd::check((x), #x)

// Grow-only device buffer (contents are not preserved on growth unless asked).
template <typename T>
struct DBuf {
  T* p = nullptr;
  size_t cap = 0;
  void ensure(size_t n, bool keep = false, size_t keep_n = 0) {
    if (n <= cap) return;
    size_t nc = cap ? cap : 1024;
    while (nc < n) nc = nc + nc / 2 + 1;
    T* np_ = nullptr;
    CK(cudaMalloc(&np_, nc * sizeof(T)));
    if (keep && p && keep_n) CK(cudaMemcpy(np_, p, keep_n * sizeof(T), cudaMemcpyDeviceToDevice));
    if (p) CK(cudaFree(p));
    p = np_;
    cap = nc;
  }
  void release() {
    if (p) cudaFree(p);
    p = nullptr;
    cap = 0;
  }
};

// Read-only geometry and state pointers passed by value to the kernels.
struct Geo;
__host__ __device__ inline bool scene_on(const Geo& g, int body);
struct Geo {
  int nb, nv, ne, nf;
  int max_prims;                        // most vertices + edges + faces of one body
  const int *v_off, *e_off, *f_off;     // nb + 1
  const double* rest;                   // nv * 3 (x, y, z per vertex)
  const int* vbody;                     // nv
  const int* ev;                        // ne * 2 global vertex ids
  const int* fv;                        // nf * 3 global vertex ids
  const double* mass;                   // nb
  const double* Ic;                     // nb
  const double* rest_box;               // nb * 6 (lo, hi), inflated by sqrt(dhat)
  const int *scene_beg, *scene_end;     // nb: body range of this body's scene
  int ns;                               // scenes (independent sub-problems of a batch)
  const int* bscene;                    // nb: scene of each body
  const int *sc_beg, *sc_end;           // ns: body range of each scene
  const double* alpha_s;                // ns or null: per-scene step for positions at q + alpha dq
  const int* sc_act;                    // ns or null: scenes to process (culls, pair terms, energies);
                                        // the others get no pairs and identity blocks
  const double *q, *dq, *q0, *dqdt;     // nb * 12
  double *X, *Xq, *X0;                  // 3 * nv, structure of arrays (x | y | z)
  double* qa;                           // nb * 12 scratch: the trial state q + alpha dq
};

__host__ __device__ inline bool scene_on(const Geo& g, int body) {
  return !g.sc_act || g.sc_act[g.bscene[body]] != 0;
}

// A culled pair set together with the overlap structure it was built on.
struct PairSet {
  int nov = 0, nnz = 0, npt = 0, nee = 0, nvg = 0;
  // symmetric overlap CSR over bodies (both (I,J) and (J,I)); upidx -> unique overlap
  DBuf<int> row_ptr, col, upidx;
  DBuf<int> ovI, ovJ;                   // unique overlaps, I < J, sorted
  DBuf<int> pt, ee;                     // 4 ints per pair: body A, prim A, body B, prim B
  DBuf<int8_t> pt_ty, ee_ty;
  DBuf<int> pt_ov, ee_ov;               // overlap of each pair
  DBuf<int> vg;                         // 2 ints per pair: body, local vertex
  DBuf<int> vg_seg;                     // nb + 1: VG pairs of each body
  // lagged friction of the pairs (valid after an assembly on this set)
  DBuf<double> pt_lag, ee_lag;          // 11 per pair, SoA: c0(3) c1(3) gamma(4) lambda
  DBuf<double> vg_lam;
};

enum { TERM_INERTIA = 1, TERM_BARRIER = 2, TERM_FRICTION = 4, TERM_ALL = 7 };
struct Params {
  double dhat, kappa, d_sqrt, eps_x, ortho_kappa, ground_offset, dt, gravity_y;
  double mu, epsv, max_uk;
  double damp_alpha, damp_beta;  // "damping": {alpha, beta}
  int psd, pt_fric, ee_fric, vg_fric, ground, pt, ee;
  int damp;                      // "damping": {enable}
  int terms;                     // TERM_* mask of the energy terms assembled (all by default)
  int exact;                     // 1: exact ground Hessian (adjoint systems)
};

// Culling scratch shared by all culls of a handle.
struct CullScratch {
  DBuf<double> bbox;
  DBuf<float> bbox_f;  // body boxes in float, rounded outward
  DBuf<int> cnt_all, cnt_up, up_ptr, rowid;
  DBuf<double> ovcull;
  DBuf<float> ovcull_f;
  DBuf<float> vbox, ebox, fbox;
  DBuf<int> order, order_cnt;           // narrow-phase processing order of the overlaps
  DBuf<int> bin_cnt, bin_off, lst;
  DBuf<long long> cand_cnt, cand_off;
  DBuf<uint8_t> flags;
  DBuf<int> blk_a, blk_b, blk_a_off, blk_b_off;
  DBuf<int> vflag_cnt, vflag_off, sub_cnt, stage_off;
  DBuf<int> vg_cnt;  // vertex-ground pairs per block of vertices
  DBuf<unsigned long long> stage_key;   // sorted accepted pairs per overlap (sub, i, j)
  DBuf<int8_t> stage_ty;
  DBuf<unsigned long long> toi_key;     // 2 per scene: pt/ee, ground
  DBuf<int> tmp_int;
  DBuf<long long> tmp_ll;
  // autotuned narrow-phase variants (index into the step table; -1 = not tuned yet) of the
  // pair cull [0] and the CCD [1], and the times measured when tuning
  int autotune = 1;
  int narrow_variant[2] = {-1, -1};
  float narrow_ms[2][3] = {{0, 0, 0}, {0, 0, 0}};
  int* h_small = nullptr;               // pinned host scratch
  long long* h_ll = nullptr;
  unsigned long long* h_toi = nullptr;
  int h_toi_cap = 0;
};

// ---------------- launch accounting ----------------
// Every kernel launch of the step goes through KLAUNCH: it counts the launch and, when
// profiling is on, brackets it with CUDA events on its stream so that each kernel's
// device time is measured live.
enum KTag {
  K_PROJECT, K_BODY_BOXES, K_OV_COUNT, K_OV_FILL, K_OV_LOWER, K_PRIM_BOXES, K_BIN, K_NARROW_SCAN,
  K_NARROW_WRITE, K_NARROW_TOI, K_VG, K_VG_TOI, K_SCAN, K_PAIR_TERMS, K_SEG, K_OV_REDUCE, K_BODY_SYSTEM,
  K_BLOCK_INVERSE, K_PCG, K_ENERGY, K_DOTS, K_VEC, K_SH, K_SORT, K_NTAGS
};
extern const char* const kTagNames[K_NTAGS];
struct Prof {
  bool on = false;
  long long launches = 0;
  double ms[K_NTAGS] = {};
  double bytes[K_NTAGS] = {};   // algorithmic bytes of the launches (per-unit figure x units)
  double units[K_NTAGS] = {};   // work units of the launches (pairs, candidates, rows, ...)
  long long cnt[K_NTAGS] = {};
  struct Rec {
    int tag;
    cudaEvent_t a, b;
  };
  std::vector<Rec> pend;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t get();
  void begin(int tag, cudaStream_t s, cudaEvent_t& a);
  void end(int tag, cudaStream_t s, cudaEvent_t a);
  void flush();  // after a stream synchronisation
  void reset();
  ~Prof();
};
extern thread_local Prof* g_prof;
inline void prof_work(int tag, double units, double bytes) {
  if (g_prof) {
    g_prof->units[tag] += units;
    g_prof->bytes[tag] += bytes;
  }
}
#define KLAUNCH(tag, stream, ...)                            \
  do {                                                      \
    cudaEvent_t _ka = nullptr;                              \
    if (::abd::g_prof) ::abd::g_prof->begin((tag), (stream), _ka); \
    __VA_ARGS__;                                            \
    CK(cudaGetLastError());                                 \
    if (::abd::g_prof) ::abd::g_prof->end((tag), (stream), _ka);   \
  } while (0)

// ---------------- scan ----------------
void scan_exclusive_int(const int* in, int* out, int n, int* d_total, cudaStream_t s, DBuf<int>& tmp);
void scan_exclusive_ll(const long long* in, long long* out, int n, long long* d_total, cudaStream_t s,
                       DBuf<long long>& tmp);

// ---------------- culling (cull.cu) ----------------
void launch_project(const Geo& g, int which, double alpha, cudaStream_t s);
// vtn 1/2: builds `out`; vtn 3: writes the per-scene TOIs (pt/ee and ground, g.ns values
// each) to toi_p and toi_g (host arrays; either may be null).
void cull(const Geo& g, const Params& P, int vtn, double alpha, CullScratch& cs, PairSet& out, double* toi_p,
          double* toi_g, cudaStream_t s);

// Line-search cull at q + alpha dq (per-scene steps of g) that reuses the overlaps and the
// refined primitive lists of the trajectory cull H of the same step (vtn 3 over q -> q + dq
// with the step not yet scaled down): the pair set equals that of a full vtn 2 cull.
void cull_trial(const Geo& g, const Params& P, double alpha, CullScratch& cs, const PairSet& H, PairSet& out,
                cudaStream_t s);

// Box-phase length of narrow-phase variant `variant` of mode 0 (pair cull) or 2 (CCD).
int narrow_step_of(int mode, int variant);

// Vertex-ground pairs (d = (y + ground_offset)^2 < P.dhat) into S.vg / S.vg_seg.
void vg_pairs(const Geo& g, const Params& P, CullScratch& cs, PairSet& S, cudaStream_t s);
void vg_count(const Geo& g, const Params& P, CullScratch& cs, cudaStream_t s);
void vg_write(const Geo& g, const Params& P, CullScratch& cs, PairSet& S, int nvg, cudaStream_t s);
// Ground times of impact of all vertices into the ground slots of the per-scene keys.
void launch_vg_toi(const Geo& g, const Params& P, unsigned long long* toi_key, cudaStream_t s);

// ---------------- sort (sort.cu) ----------------
size_t sort_padded_size(size_t n);  // buffer size sort_u64 needs for n keys
void sort_u64(unsigned long long* keys, size_t n, size_t cap, cudaStream_t s);

// ---------------- spatial-hash broad phase (shash.cu) ----------------
struct ShParams {
  double min_xyz, dx, safe_factor;
  int bits, fix_edge, full_ccd;
};
struct ShTable {
  DBuf<long long> cnt, off, scan_tmp;
  DBuf<unsigned long long> keys;
  DBuf<int> bstart, bend;
  long long n = 0;
  long long h_tot = 0;
};
struct ShScratch {
  ShTable tab;
  DBuf<int> qcnt, qoff, scan_i, flag, pos;
  DBuf<unsigned long long> pt_keys, ee_keys, bp_all, tkeys;
  DBuf<unsigned> bp_pt, bp_ee;
  int* h_int = nullptr;
  unsigned long long* h_toi = nullptr;
  int h_toi_cap = 0;
};
// gen_collision_set: pair set of the configuration at q (vtn 1) or q + alpha dq (vtn 2).
void sh_cull(const Geo& g, const Params& P, const ShParams& H, int vtn, double alpha, ShScratch& W, CullScratch& cs,
             PairSet& S, cudaStream_t s);
// step_size_upper_bound: per-scene bound of the step q -> q + dq into toi (host, g.ns).
void sh_bound(const Geo& g, const Params& P, const ShParams& H, const PairSet& cur, ShScratch& W, CullScratch& cs,
              double* toi, cudaStream_t s);

// ---------------- Newton system (newton.cu) ----------------
enum { CONTRIB = 456 };  // dI(144) dJ(144) off(144) gI(12) gJ(12)
struct NewtonBufs {
  DBuf<double> pt_c, ee_c;   // CONTRIB per pair (SoA)
  DBuf<int> pt_seg, ee_seg;  // nov + 1
  DBuf<int> perm, cls_cnt, cls_off, cls_tmp;  // pairs in distance-type order
  DBuf<double> prec;         // per-pair reduced Hessian records between the pair-term kernels
  cudaStream_t side = nullptr;               // mollified pairs run beside the main pair kernel
  cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
  DBuf<double> ovr;          // nov * CONTRIB
  DBuf<int> has;             // nov
  DBuf<double> D, Dinv, grad;
  DBuf<double> x, r, z, p, qv;   // p: two buffers (iteration parity)
  DBuf<double> Hrow;         // row-block copy of the system for the PCG
  DBuf<int> rcol, rn;
  DBuf<double> gpA, gpB;     // per-group partial sums of the PCG
  DBuf<int> grp_body, grp_n, grp_scene, sc_gbeg, sc_gend;  // PCG body groups (pcg_groups)
  std::vector<int> h_sc_beg, h_sc_end;  // body range of each scene (host)
  DBuf<double> dense_A, dense_y;         // dense solve: one scene's matrix and right-hand side
  // block-tridiagonal direct solve: per-scene flags and counts, per-body link to the next
  // body, the factor's inverse diagonal blocks, coupling blocks and forward solution
  DBuf<int> tri_bad, tri_on, pcg_on, tri_cnt, tri_link;
  DBuf<double> tri_Li, tri_W, tri_y;
  // adjoint: friction-frame Jacobians and contributions per pair, the exact system's
  // blocks, GMRES bases
  DBuf<double> fj_pt, fj_ee, fc_pt, fc_ee, D_ex, ovr_ex, adj_V, adj_Z, adj_w, adj_t, adj_x;
  DBuf<int> has_ex;
  double* h_dot = nullptr;               // pinned: one dot product
  int ngrp = 0;
  DBuf<double> sc_rz, sc_bb; // per-scene CG scalars
  DBuf<int> sc_conv, sc_iters, n_active;
  DBuf<double> red;          // chunk partial sums of the energies
  DBuf<int> e_off, e_chunk_cnt, e_chunk_off, e_scan_tmp;
  DBuf<double> e_out;        // per-scene energies / dot products
  DBuf<int> status;          // [0] solver status, [1] pcg iters
  DBuf<double> xr, rt, dqc;  // iterative refinement: accumulated solution, true residual, -d
  DBuf<int> it_ref;          // refinement: [0] total iterations, [2 + k] per scene
  std::vector<int> h_ref;
  double* h_red = nullptr;   // pinned
  int* h_int = nullptr;
};
void assemble(const Geo& g, const Params& P, PairSet& S, NewtonBufs& nb, cudaStream_t s);
// Solves H x = grad per scene (scenes with sc_on[s] == 0 get x = 0); dq = -x. Returns the
// iterations of the longest scene; scene_iters (host, ns) receives each scene's count.
// Body groups of the PCG (consecutive bodies of one scene, cut from the scene's first
// body); called once per handle with the scenes' body ranges.
void pcg_groups(const std::vector<int>& sc_beg, const std::vector<int>& sc_end, NewtonBufs& nb, cudaStream_t s);
// Newton-solve controls: PCG relative residual and iteration cap; refine > 0: that many
// iterative-refinement passes, each solving H d = b - H x (true residual) by the same PCG
// to refine_tol relative and adding d to x; dense: a dense Cholesky per scene instead of
// the PCG (the reference's "solver": "dense").
struct SolveOpts {
  double rel_tol = 1e-14;
  int max_iter = 5000;
  int refine = 0;
  double refine_tol = 1e-8;
  int dense = 0;
  int tri = 0;  // block-tridiagonal scenes by block Cholesky (tri_solve)
};
// on (host, ns): the scenes solved (the others get dq = 0); sc_on is its device copy.
int pcg_solve(const Geo& g, PairSet& S, NewtonBufs& nb, const SolveOpts& o, const int* sc_on,
              const std::vector<char>& on, double* dq, cudaStream_t s, int* status, int* scene_iters);
// Block-tridiagonal scenes (tri.cu; after the row-block copy of pcg_solve): tri_classify
// marks the scenes whose blocks only join consecutive bodies (tri_on, when enable) and the
// others solved (pcg_on), returning both counts; tri_solve factorizes and solves every run
// of linked bodies of the tri_on scenes (x, dq = -x) and writes x = 0, dq = -0 for the
// scenes with sc_on == 0.
void tri_classify(const Geo& g, PairSet& S, NewtonBufs& B, int enable, const int* sc_on, cudaStream_t s,
                  int* n_pcg, int* n_tri);
void tri_solve(const Geo& g, PairSet& S, NewtonBufs& B, const int* sc_on, double* dq, cudaStream_t s);
// Dense Cholesky solve of each scene's system (after the row-block copy of pcg_solve).
void dense_solve(const Geo& g, PairSet& S, NewtonBufs& B, const std::vector<char>& on, double* dq, cudaStream_t s);
// Line-search energy of every scene at the trial configuration (X must hold q + alpha dq):
// inertia + barrier over `Snew` + lagged friction over `Slag`; out (host) receives ns values.
void energy(const Geo& g, const Params& P, double alpha, PairSet& Snew, PairSet& Slag, bool with_barrier_inertia,
            NewtonBufs& nb, cudaStream_t s, double* out);
// Every term of that energy on its own, into device array `out`: the bodies' inertia +
// orthogonality (nb), the barrier energies of Snew's PT, EE, VG pairs, then the friction
// energies of Slag's PT, EE, VG pairs, in list order.
void energy_terms(const Geo& g, const Params& P, double alpha, PairSet& Snew, PairSet& Slag, double* out,
                  cudaStream_t s);
// Per scene over its 12 n dofs: out[3s] = dq.grad, out[3s+1] = |grad|^2, out[3s+2] = |dq|^2
void dots(const Geo& g, const double* dq, const double* grad, NewtonBufs& nb, double* out, cudaStream_t s);
// Per scene: out[3s] = a.b, out[3s+1] = |b|^2, out[3s+2] = |a - b|^2
void scene_diff(const Geo& g, const double* a, const double* b, NewtonBufs& nb, double* out, cudaStream_t s);
void launch_copy_scene(const Geo& g, double* dst, const double* src, const int* on, cudaStream_t st);
void launch_scale_scene(const Geo& g, double* v, const double* f, cudaStream_t st);
// y = H x with the system assembled last on S (no synchronisation)
void spmv(const Geo& g, const PairSet& S, NewtonBufs& nb, const double* x, double* y, cudaStream_t st);
// y = H x with explicitly given blocks (saved copies of an assembly on S)
void spmv_blocks(const Geo& g, const PairSet& S, const int* has, const double* ovr, const double* D, const double* x,
                 double* y, cudaStream_t st);
// ---------------- adjoint (adjoint.cu) ----------------
// Per PT/EE pair of S: the Jacobian of its friction force through its tangent frame and
// multiplier at the positions in g.X (reference positions g.X0), kept in B.fj_pt / fj_ee.
void fric_frame_jacobians(const Geo& g, const Params& P, PairSet& S, NewtonBufs& B, cudaStream_t s);
// out = (those Jacobians, in body coordinates)^T w, summed per body in a fixed order
// (needs the overlap segments of the last assembly on S).
void fric_frame_apply_t(const Geo& g, PairSet& S, NewtonBufs& B, const double* w, double* out, cudaStream_t s);
double dev_dot(int n, const double* a, const double* b, NewtonBufs& B, cudaStream_t s);  // synchronises
void dev_axpby(int n, double a, const double* x, double b, double* y, cudaStream_t s);   // y = a x + b y
// out = C^T w for the ground-friction multiplier coupling of an adjoint system
void vg_lag_adjoint(const Geo& g, const Params& P, const PairSet& S, const double* w, double* out, cudaStream_t st);
void launch_q_update_scene(const Geo& g, double* q, const double* dq, const double* alpha, cudaStream_t st);
void launch_frame_end(double* q, double* q0, double* dqdt, int n, double dt, cudaStream_t st);
void launch_copy(double* dst, const double* src, int n, cudaStream_t st);

// ---------------- per-primitive batches (prims.cu) ----------------
double measure_fp64_gflops();

}  // namespace abd
