// Host side of the GB300 step: the handle, its device buffers, the per-frame Newton
// loop (the reference's ABD::implicit_euler, model/abd.cpp:30-140, with ccd() :142-196
// and line_search(dt) :198-227 / model/line_search.cpp:39-136) and the C ABI.
#include <chrono>
#include <cmath>
#include <cstring>
#include <stdexcept>
#include <string>
#include <unordered_set>
#include <vector>

#include "abd_engine.h"

namespace abd {

void check(cudaError_t e, const char* where) {
  if (e != cudaSuccess) throw CudaError{e, where};
}

const char* const kTagNames[K_NTAGS] = {
    "project", "body_boxes", "ov_count", "ov_fill", "ov_lower", "prim_boxes", "bin", "narrow_scan",
    "narrow_write", "narrow_toi", "vg", "vg_toi", "scan", "pair_terms", "seg", "ov_reduce", "body_system",
    "block_inverse", "pcg", "energy", "dots", "vec", "spatial_hash", "sort"};
thread_local Prof* g_prof = nullptr;

cudaEvent_t Prof::get() {
  if (!pool.empty()) {
    cudaEvent_t e = pool.back();
    pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  CK(cudaEventCreate(&e));
  return e;
}
void Prof::begin(int tag, cudaStream_t s, cudaEvent_t& a) {
  (void)tag;
  ++launches;
  if (!on) return;
  a = get();
  CK(cudaEventRecord(a, s));
}
void Prof::end(int tag, cudaStream_t s, cudaEvent_t a) {
  if (!on || !a) return;
  cudaEvent_t b = get();
  CK(cudaEventRecord(b, s));
  pend.push_back(Rec{tag, a, b});
}
void Prof::flush() {
  for (auto& r : pend) {
    CK(cudaEventSynchronize(r.b));
    float t = 0;
    CK(cudaEventElapsedTime(&t, r.a, r.b));
    ms[r.tag] += t;
    cnt[r.tag] += 1;
    pool.push_back(r.a);
    pool.push_back(r.b);
  }
  pend.clear();
}
void Prof::reset() {
  flush();
  for (int i = 0; i < K_NTAGS; ++i) {
    ms[i] = 0;
    cnt[i] = 0;
    bytes[i] = 0;
    units[i] = 0;
  }
  launches = 0;
}
Prof::~Prof() {
  for (auto& r : pend) {
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  for (auto e : pool) cudaEventDestroy(e);
}

struct Engine {
  abd_config cfg;
  Params P;
  int nb = 0, nv = 0, ne = 0, nf = 0;
  int max_prims = 0;                             // most vertices + edges + faces of one body
  cudaStream_t s = nullptr;
  DBuf<int> v_off, e_off, f_off, vbody, ev, fv, scene_beg, scene_end;
  DBuf<double> rest, mass, Ic, rest_box, q, q0, dqdt, dq, X, Xq, X0, lastdq, qa;
  PairSet sets[3];
  int cur = 0;
  CullScratch cs;
  NewtonBufs nbufs;
  int last_cull_set = 0;
  // scenes: independent sub-problems, each with its own Newton loop, step bound and
  // line search (a single scene is the reference's ABD::implicit_euler)
  int ns = 1;
  DBuf<int> bscene, sc_beg, sc_end, sc_on, sc_iter, sc_search;
  DBuf<double> sc_alpha, sc_factor;
  std::vector<int> h_sc_beg, h_sc_end;
  std::vector<int> iter, g_cnt, p_cnt;           // per scene (iter: cumulative, model/abd.h:53)
  std::vector<int> sc_newton, sc_ls, sc_pcg;     // per scene, over the last abd_step call
  std::vector<char> has_lastdq;                  // per scene: lastdq holds a previous step
  ShParams sh{};                                 // spatial-hash broad phase (iaabb even / <= 1)
  ShScratch shw;
  int* h_on = nullptr;                           // pinned staging of per-scene uploads
  int *h_iter = nullptr, *h_search = nullptr;
  double *h_alpha = nullptr, *h_factor = nullptr;
  std::string err;
  Prof prof;
  // trace settings of the reference's viewer loop (view/control.cpp:41,84-90;
  // view/model_view.cpp:282-295): frame counter, last frame, folder, and the config and
  // scene files copied into a new trace folder
  int ts = 0, starting_ts = -1, ending_ts = 0;
  int adj_iters = 0;            // GMRES iterations of the last abd_adjoint_frame
  double adj_residual = 0.0;    // its final relative residual (restart estimate)
  std::string trace_folder = "trace", trace_config, trace_scene;

  Geo geo() const {
    Geo g;
    g.nb = nb; g.nv = nv; g.ne = ne; g.nf = nf; g.max_prims = max_prims;
    g.v_off = v_off.p; g.e_off = e_off.p; g.f_off = f_off.p;
    g.rest = rest.p; g.vbody = vbody.p; g.ev = ev.p; g.fv = fv.p;
    g.mass = mass.p; g.Ic = Ic.p; g.rest_box = rest_box.p;
    g.scene_beg = scene_beg.p; g.scene_end = scene_end.p;
    g.ns = ns; g.bscene = bscene.p; g.sc_beg = sc_beg.p; g.sc_end = sc_end.p; g.alpha_s = nullptr;
    g.sc_act = nullptr;
    g.q = q.p; g.dq = dq.p; g.q0 = q0.p; g.dqdt = dqdt.p;
    g.X = X.p; g.Xq = Xq.p; g.X0 = X0.p; g.qa = qa.p;
    return g;
  }

  ~Engine() {
    DBuf<int>* ib[] = {&v_off,  &e_off,  &f_off,  &vbody, &ev,    &fv,      &scene_beg, &scene_end,
                       &bscene, &sc_beg, &sc_end, &sc_on, &sc_iter, &sc_search};
    for (auto* b : ib) b->release();
    DBuf<double>* db[] = {&rest, &mass, &Ic, &rest_box, &q, &q0, &dqdt, &dq, &X, &Xq, &X0, &sc_alpha, &sc_factor,
                          &lastdq, &qa};
    for (auto* b : db) b->release();
    for (auto& S : sets) {
      S.row_ptr.release(); S.col.release(); S.upidx.release(); S.ovI.release(); S.ovJ.release();
      S.pt.release(); S.ee.release(); S.pt_ty.release(); S.ee_ty.release(); S.pt_ov.release(); S.ee_ov.release();
      S.vg.release(); S.vg_seg.release(); S.pt_lag.release(); S.ee_lag.release(); S.vg_lam.release();
    }
    cs.bbox.release(); cs.bbox_f.release(); cs.cnt_all.release(); cs.cnt_up.release(); cs.up_ptr.release(); cs.rowid.release();
    cs.ovcull.release(); cs.ovcull_f.release(); cs.vbox.release(); cs.ebox.release(); cs.fbox.release();
    cs.order.release(); cs.order_cnt.release();
    cs.bin_cnt.release(); cs.bin_off.release(); cs.lst.release(); cs.cand_cnt.release(); cs.cand_off.release();
    cs.flags.release(); cs.blk_a.release(); cs.blk_b.release(); cs.blk_a_off.release(); cs.blk_b_off.release();
    cs.vflag_cnt.release(); cs.vflag_off.release(); cs.sub_cnt.release(); cs.stage_off.release(); cs.vg_cnt.release();
    cs.stage_key.release(); cs.stage_ty.release(); cs.toi_key.release(); cs.tmp_int.release(); cs.tmp_ll.release();
    if (cs.h_small) cudaFreeHost(cs.h_small);
    if (cs.h_ll) cudaFreeHost(cs.h_ll);
    if (cs.h_toi) cudaFreeHost(cs.h_toi);
    nbufs.pt_c.release(); nbufs.ee_c.release(); nbufs.pt_seg.release(); nbufs.ee_seg.release();
    nbufs.ovr.release(); nbufs.has.release(); nbufs.D.release(); nbufs.Dinv.release(); nbufs.grad.release();
    nbufs.x.release(); nbufs.r.release(); nbufs.z.release(); nbufs.p.release(); nbufs.qv.release();
    nbufs.Hrow.release(); nbufs.rcol.release(); nbufs.rn.release();
    nbufs.perm.release(); nbufs.cls_cnt.release(); nbufs.cls_off.release(); nbufs.cls_tmp.release();
    nbufs.prec.release();
    if (nbufs.side) cudaStreamDestroy(nbufs.side);
    if (nbufs.ev_fork) cudaEventDestroy(nbufs.ev_fork);
    if (nbufs.ev_join) cudaEventDestroy(nbufs.ev_join);
    nbufs.gpA.release(); nbufs.gpB.release(); nbufs.grp_body.release(); nbufs.grp_n.release();
    nbufs.grp_scene.release(); nbufs.sc_gbeg.release(); nbufs.sc_gend.release(); nbufs.sc_rz.release(); nbufs.sc_bb.release();
    nbufs.sc_conv.release(); nbufs.sc_iters.release(); nbufs.n_active.release();
    nbufs.e_off.release(); nbufs.e_chunk_cnt.release(); nbufs.e_chunk_off.release(); nbufs.e_scan_tmp.release();
    nbufs.e_out.release(); nbufs.red.release(); nbufs.status.release();
    nbufs.xr.release(); nbufs.rt.release(); nbufs.dqc.release(); nbufs.it_ref.release();
    nbufs.dense_A.release(); nbufs.dense_y.release();
    nbufs.fj_pt.release(); nbufs.fj_ee.release(); nbufs.fc_pt.release(); nbufs.fc_ee.release();
    nbufs.D_ex.release(); nbufs.ovr_ex.release(); nbufs.has_ex.release(); nbufs.adj_V.release();
    nbufs.adj_Z.release(); nbufs.adj_w.release(); nbufs.adj_t.release(); nbufs.adj_x.release();
    if (nbufs.h_dot) cudaFreeHost(nbufs.h_dot);
    if (nbufs.h_red) cudaFreeHost(nbufs.h_red);
    if (nbufs.h_int) cudaFreeHost(nbufs.h_int);
    if (h_on) cudaFreeHost(h_on);
    if (h_iter) cudaFreeHost(h_iter);
    if (h_search) cudaFreeHost(h_search);
    if (h_alpha) cudaFreeHost(h_alpha);
    if (h_factor) cudaFreeHost(h_factor);
    if (s) cudaStreamDestroy(s);
  }

  template <typename T>
  void upload(DBuf<T>& b, const T* src, size_t n) {
    b.ensure(n ? n : 1);
    if (n) CK(cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice, s));
  }

  void init(const abd_scene_desc* d, const abd_config* c) {
    cfg = *c;
    P.dhat = c->dhat;
    P.kappa = c->kappa;
    P.d_sqrt = std::sqrt(c->dhat);
    P.eps_x = c->eps_x;
    P.ortho_kappa = c->ortho_kappa;
    P.ground_offset = c->ground_offset;
    P.dt = c->dt;
    P.gravity_y = c->gravity_y;
    P.mu = c->mu;
    P.epsv = c->dt * c->evh;
    P.max_uk = c->max_uk;
    P.psd = c->psd;
    P.pt_fric = c->pt_fric;
    P.ee_fric = c->ee_fric;
    P.vg_fric = c->vg_fric;
    P.ground = c->ground;
    P.pt = c->pt;
    P.ee = c->ee;
    P.terms = TERM_ALL;
    P.exact = 0;
    P.damp = c->damping;
    P.damp_alpha = c->damp_alpha;
    P.damp_beta = c->damp_beta;
    sh.min_xyz = c->sh_min_xyz;
    sh.dx = c->sh_dx;
    sh.safe_factor = c->safe_factor;
    sh.bits = c->sh_xyz_bits;
    sh.fix_edge = c->sh_fix_edge_trajectory;
    sh.full_ccd = c->full_ccd;
    if (c->iaabb % 2 == 0 || (c->upper_bound && c->iaabb <= 1)) {
      if (!(c->sh_dx > 0) || c->sh_xyz_bits < 1 || c->sh_xyz_bits > 9 || !(c->safe_factor > 0))
        throw std::invalid_argument("spatial hashing: need dx > 0, 1 <= xyz_bits <= 9, safe_factor > 0");
    }
    if (c->iaabb % 2 == 0) {
      // the reference's hash entries hold 16-bit body and primitive ids (spatial_hashing.h:9)
      bool ok = d->n_bodies <= 32767;
      for (int b = 0; ok && b < d->n_bodies; ++b)
        ok = d->vert_off[b + 1] - d->vert_off[b] <= 32767 && d->edge_off[b + 1] - d->edge_off[b] <= 32767 &&
             d->face_off[b + 1] - d->face_off[b] <= 32767;
      if (!ok) throw std::invalid_argument("spatial hashing: at most 32767 bodies and 32767 primitives per body");
    }
    cs.autotune = c->autotune;
    CK(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
    nb = d->n_bodies;
    nv = d->vert_off[nb];
    ne = d->edge_off[nb];
    nf = d->face_off[nb];
    std::vector<int> hvb(nv), hev(2 * (size_t)ne), hfv(3 * (size_t)nf), sb(nb), se(nb);
    std::vector<double> rb(6 * (size_t)nb);
    for (int b = 0; b < nb; ++b) {
      int np = (d->vert_off[b + 1] - d->vert_off[b]) + (d->edge_off[b + 1] - d->edge_off[b]) +
               (d->face_off[b + 1] - d->face_off[b]);
      max_prims = np > max_prims ? np : max_prims;
      for (int v = d->vert_off[b]; v < d->vert_off[b + 1]; ++v) hvb[v] = b;
      for (int e = d->edge_off[b]; e < d->edge_off[b + 1]; ++e)
        for (int k = 0; k < 2; ++k) {
          int lv = d->edges[2 * e + k];
          if (lv < 0 || lv >= d->vert_off[b + 1] - d->vert_off[b]) throw std::invalid_argument("edge vertex id");
          hev[2 * e + k] = d->vert_off[b] + lv;
        }
      for (int f = d->face_off[b]; f < d->face_off[b + 1]; ++f)
        for (int k = 0; k < 3; ++k) {
          int lv = d->faces[3 * f + k];
          if (lv < 0 || lv >= d->vert_off[b + 1] - d->vert_off[b]) throw std::invalid_argument("face vertex id");
          hfv[3 * f + k] = d->vert_off[b] + lv;
        }
      // rest AABB inflated by sqrt(dhat) (iaabb.cpp:23-39)
      double lo[3], hi[3];
      for (int v = d->vert_off[b]; v < d->vert_off[b + 1]; ++v)
        for (int k = 0; k < 3; ++k) {
          double x = d->rest_vertices[3 * v + k];
          if (v == d->vert_off[b]) lo[k] = hi[k] = x;
          else {
            lo[k] = x < lo[k] ? x : lo[k];
            hi[k] = hi[k] < x ? x : hi[k];
          }
        }
      for (int k = 0; k < 3; ++k) {
        rb[6 * b + k] = lo[k] - P.d_sqrt;
        rb[6 * b + 3 + k] = hi[k] + P.d_sqrt;
      }
    }
    // scene ranges (bodies of a scene are contiguous)
    std::vector<int> hbs(nb);
    std::unordered_set<int> seen;
    h_sc_beg.clear();
    h_sc_end.clear();
    for (int b = 0; b < nb;) {
      int e = b + 1;
      if (d->scene_id)
        while (e < nb && d->scene_id[e] == d->scene_id[b]) ++e;
      else
        e = nb;
      if (d->scene_id && !seen.insert(d->scene_id[b]).second)
        throw std::invalid_argument("bodies of a scene must be contiguous");
      for (int k = b; k < e; ++k) {
        sb[k] = b;
        se[k] = e;
        hbs[k] = (int)h_sc_beg.size();
      }
      h_sc_beg.push_back(b);
      h_sc_end.push_back(e);
      b = e;
    }
    ns = (int)h_sc_beg.size();
    iter.assign(ns, 0);
    g_cnt.assign(ns, 0);
    p_cnt.assign(ns, 0);
    sc_newton.assign(ns, 0);
    sc_ls.assign(ns, 0);
    sc_pcg.assign(ns, 0);
    CK(cudaMallocHost(&h_on, ns * sizeof(int)));
    CK(cudaMallocHost(&h_iter, ns * sizeof(int)));
    CK(cudaMallocHost(&h_search, ns * sizeof(int)));
    sc_iter.ensure(ns);
    sc_search.ensure(ns);
    CK(cudaMallocHost(&h_alpha, ns * sizeof(double)));
    CK(cudaMallocHost(&h_factor, ns * sizeof(double)));
    upload(bscene, hbs.data(), nb);
    upload(sc_beg, h_sc_beg.data(), ns);
    upload(sc_end, h_sc_end.data(), ns);
    abd::pcg_groups(h_sc_beg, h_sc_end, nbufs, s);
    sc_on.ensure(ns);
    sc_alpha.ensure(ns);
    sc_factor.ensure(ns);
    upload(v_off, d->vert_off, nb + 1);
    upload(e_off, d->edge_off, nb + 1);
    upload(f_off, d->face_off, nb + 1);
    upload(vbody, hvb.data(), nv);
    upload(ev, hev.data(), 2 * (size_t)ne);
    upload(fv, hfv.data(), 3 * (size_t)nf);
    upload(scene_beg, sb.data(), nb);
    upload(scene_end, se.data(), nb);
    upload(rest, d->rest_vertices, 3 * (size_t)nv);
    upload(mass, d->mass, nb);
    upload(Ic, d->Ic, nb);
    upload(rest_box, rb.data(), 6 * (size_t)nb);
    upload(q0, d->q0, 12 * (size_t)nb);
    upload(q, d->q0, 12 * (size_t)nb);
    upload(dqdt, d->dqdt, 12 * (size_t)nb);
    dq.ensure(12 * (size_t)nb);
    CK(cudaMemsetAsync(dq.p, 0, 12 * (size_t)nb * sizeof(double), s));
    lastdq.ensure(12 * (size_t)nb);
    CK(cudaMemsetAsync(lastdq.p, 0, 12 * (size_t)nb * sizeof(double), s));
    has_lastdq.assign(ns, 0);
    X.ensure(3 * (size_t)nv + 3);
    Xq.ensure(3 * (size_t)nv + 3);
    qa.ensure(12 * (size_t)nb + 12);
    X0.ensure(3 * (size_t)nv + 3);
    CK(cudaStreamSynchronize(s));
  }

  // Algorithmic bytes of the path (per-stage formula, from logged counts).
  double bytes_cull(const PairSet& S) const {
    return 48.0 * nv + 24.0 * nv + 20.0 * (S.npt + S.nee + S.nvg);
  }
  double bytes_assemble(const PairSet& S) const {
    double P_ = S.npt + S.nee;
    return (20 + 96 + 96) * P_ + 200 * P_ + 2 * 1152.0 * (nb + 2.0 * S.nov) + 2 * 96.0 * nb;
  }

  // Pair-set culling at q (vtn 1) or at q + alpha dq (vtn 2): iAABB for odd iaabb, the
  // spatial hash for even (abd.cpp:48-51, line_search.cpp:88-110).
  // Positions at q + alpha dq use the per-scene steps of g when it carries them.
  void cull_set(const Geo& g, int vtn, PairSet& S, double alpha = 1.0) {
    if (cfg.iaabb % 2) cull(g, P, vtn, alpha, cs, S, nullptr, nullptr, s);
    else sh_cull(g, P, sh, vtn, alpha, shw, cs, S, s);
  }

  SolveOpts solve_opts() const {
    SolveOpts o;
    o.rel_tol = cfg.pcg_rel_tol;
    o.max_iter = cfg.pcg_max_iter;
    o.refine = cfg.pcg_refine;
    o.refine_tol = cfg.pcg_refine_tol;
    o.dense = cfg.solver == 1;
    o.tri = cfg.tri_direct;
    return o;
  }

  // Uploads of per-scene values go through pinned staging arrays; every upload is followed
  // by a stream synchronisation before its staging array is written again.
  void put_on(const std::vector<char>& on) {
    for (int k = 0; k < ns; ++k) h_on[k] = on[k] ? 1 : 0;
    CK(cudaMemcpyAsync(sc_on.p, h_on, ns * sizeof(int), cudaMemcpyHostToDevice, s));
  }
  // masks of the scenes still iterating / still searching (culls, pair terms, energies)
  void put_mask(DBuf<int>& d, int* h, const std::vector<char>& on) {
    for (int k = 0; k < ns; ++k) h[k] = on[k] ? 1 : 0;
    CK(cudaMemcpyAsync(d.p, h, ns * sizeof(int), cudaMemcpyHostToDevice, s));
  }
  void put_alpha(const std::vector<double>& a) {
    for (int k = 0; k < ns; ++k) h_alpha[k] = a[k];
    CK(cudaMemcpyAsync(sc_alpha.p, h_alpha, ns * sizeof(double), cudaMemcpyHostToDevice, s));
  }
  void put_factor(const std::vector<double>& f) {
    for (int k = 0; k < ns; ++k) h_factor[k] = f[k];
    CK(cudaMemcpyAsync(sc_factor.p, h_factor, ns * sizeof(double), cudaMemcpyHostToDevice, s));
  }

  // One frame of every scene. Each scene follows ABD::implicit_euler on its own: Newton
  // iterations until its own |dq| < tol (or its own counter reaches max_iter), its own
  // CCD bound and its own Armijo line search; a scene that has finished keeps its state
  // while the others iterate (its dq is 0). With one scene this is the reference loop.
  int step_frame(abd_frame_stats& st) {
    using clk = std::chrono::steady_clock;
    auto ms = [](clk::time_point a, clk::time_point b) {
      return std::chrono::duration<double, std::milli>(b - a).count();
    };
    Geo g = geo();
    const int n12 = 12 * nb;
    launch_copy(q.p, q0.p, n12, s);
    CK(cudaMemsetAsync(dq.p, 0, n12 * sizeof(double), s));
    launch_project(g, 0, 0.0, s);
    cull_set(g, 1, sets[cur]);
    st.bytes_moved += bytes_cull(sets[cur]);
    std::vector<char> act(ns, 1), ls(ns, 0), stalled(ns, 0);
    std::vector<double> dd(3 * ns), sup_dq(ns), tp(ns, 1.0), tg(ns, 1.0), toi(ns, 1.0), fac(ns, 1.0);
    std::vector<double> E0(ns), E1(ns), qdg(ns), gn(ns), dqn(ns), a_cull(ns, 1.0), a_fin(ns, 1.0);
    std::vector<int> trials(ns, 0), its_s(ns, 0), fin_pass(ns, 0), its_f(ns, 0);
    int n_act = ns;
    int status = ABD_OK;
    while (n_act > 0) {
      auto t0 = clk::now();
      PairSet& S = sets[cur];
      put_mask(sc_iter, h_iter, act);
      Geo ga = g;  // the scenes still iterating
      ga.sc_act = sc_iter.p;
      st.n_pt = std::max(st.n_pt, S.npt);
      st.n_ee = std::max(st.n_ee, S.nee);
      st.n_vg = std::max(st.n_vg, S.nvg);
      st.n_overlaps = std::max(st.n_overlaps, S.nov);
      assemble(ga, P, S, nbufs, s);
      put_on(act);
      st.bytes_moved += bytes_assemble(S);
      auto t1 = clk::now();
      int pst = 0;
      int its = pcg_solve(g, S, nbufs, solve_opts(), sc_on.p, act, dq.p, s, &pst, its_s.data());
      st.pcg_iters += its;
      for (int k = 0; k < ns; ++k) sc_pcg[k] += its_s[k];
      // N_blk = bodies + 2 x contacting body pairs: the blocks the PCG keeps (nbufs.h_int[2])
      st.bytes_moved += its * (1152.0 * nbufs.h_int[2] + 6 * 96.0 * nb) + 1152.0 * nb;
      if (pst == ABD_ERR_NOT_SPD) return ABD_ERR_NOT_SPD;
      if (pst == ABD_ERR_PCG_NOCONV) status = ABD_ERR_PCG_NOCONV;
      dots(g, dq.p, nbufs.grad.p, nbufs, dd.data(), s);
      for (int k = 0; k < ns; ++k) {
        sup_dq[k] = std::sqrt(dd[3 * k + 2]);
        if (act[k] && std::isnan(sup_dq[k])) return ABD_ERR_NAN;
      }
      auto t2 = clk::now();
      // CCD step bound (abd.cpp:142-196)
      for (int k = 0; k < ns; ++k) toi[k] = 1.0;
      bool hull = false;  // the iAABB trajectory cull of this step can serve the trial culls
      if (cfg.upper_bound && cfg.iaabb <= 1) {
        // step_size_upper_bound (upper_bound.cpp:16-277)
        sh_bound(ga, P, sh, S, shw, cs, toi.data(), s);
        st.bytes_moved += 96.0 * nv;
      } else if (cfg.upper_bound) {
        cull(ga, P, 3, 1.0, cs, sets[2], tp.data(), tg.data(), s);
        hull = cfg.iaabb % 2 == 1;
        st.bytes_moved += 96.0 * nv + 20.0 * sets[2].nov;
        for (int k = 0; k < ns; ++k) {
          if (!act[k]) continue;
          if (cfg.ground) {
            if (tg[k] < 1e-6) g_cnt[k]++;
            else g_cnt[k] = 0;
          }
          if (tp[k] < 1e-6) p_cnt[k]++;
          else p_cnt[k] = 0;
          toi[k] = cfg.ground ? std::min(tg[k], tp[k]) : tp[k];
          if ((cfg.ground && g_cnt[k] > 1) || p_cnt[k] > 1) return ABD_ERR_TOI_TINY;
        }
      }
      // same-direction stop (abd.cpp:180-190): with dq_tol <= 0 it can never trigger
      if (cfg.dq_tol > 0) {
        std::vector<double> df(3 * ns);
        scene_diff(g, dq.p, lastdq.p, nbufs, df.data(), s);
        for (int k = 0; k < ns; ++k) {
          if (!act[k] || !iter[k] || !has_lastdq[k]) continue;
          double c = df[3 * k] / (std::sqrt(dd[3 * k + 2]) * std::sqrt(df[3 * k + 1]));
          if (std::fabs(c) > 1.0 - cfg.dq_tol && std::sqrt(df[3 * k + 2]) / std::sqrt(dd[3 * k + 2]) < cfg.dq_tol)
            return ABD_ERR_SAME_DIRECTION;
        }
        launch_copy_scene(g, lastdq.p, dq.p, sc_on.p, s);
        for (int k = 0; k < ns; ++k)
          if (act[k]) has_lastdq[k] = 1;
      }
      for (int k = 0; k < ns; ++k) {
        double factor = toi[k] < 1.0 ? cfg.backoff : 1.0;
        fac[k] = factor * toi[k];
        if (act[k]) st.toi_min = std::min(st.toi_min, toi[k]);
      }
      put_factor(fac);
      launch_scale_scene(g, dq.p, sc_factor.p, s);
      auto t3 = clk::now();
      // line search (line_search.cpp:39-136), all scenes' trials in one culling pass
      for (int k = 0; k < ns; ++k) a_fin[k] = act[k] ? 1.0 : 0.0;
      if (cfg.line_search) {
        launch_project(g, 1, 0.0, s);
        energy(ga, P, 0.0, S, S, true, nbufs, s, E0.data());
        dots(g, dq.p, nbufs.grad.p, nbufs, dd.data(), s);
        for (int k = 0; k < ns; ++k) {
          qdg[k] = dd[3 * k];
          gn[k] = std::sqrt(dd[3 * k + 1]);
          dqn[k] = std::sqrt(dd[3 * k + 2]);
          ls[k] = act[k];
          stalled[k] = act[k];
          trials[k] = 0;
          a_cull[k] = act[k] ? 1.0 : 0.0;
        }
        int other = 1 - cur;
        int n_ls = n_act;
        Geo gt = g;  // trial positions of the scenes still searching
        gt.alpha_s = sc_alpha.p;
        gt.sc_act = sc_search.p;
        int pass = 0, early = 0;  // early: scenes that finished before the last pass
        while (n_ls > 0) {
          put_mask(sc_search, h_search, ls);
          put_alpha(a_cull);
          // trial positions lie on the trajectory the CCD culled: its broad phase is reused
          if (hull) cull_trial(gt, P, 1.0, cs, sets[2], sets[other], s);
          else cull_set(gt, 2, sets[other]);
          energy(gt, P, 0.0, sets[other], S, true, nbufs, s, E1.data());
          ++pass;
          st.bytes_moved += bytes_cull(sets[other]) + 48.0 * nv + 116.0 * (sets[other].npt + sets[other].nee);
          for (int k = 0; k < ns; ++k) {
            if (!ls[k]) continue;
            ++trials[k];
            bool wolfe = E1[k] <= E0[k] + cfg.c1 * a_cull[k] * qdg[k];
            double alpha = a_cull[k] / 2;
            bool done = false;
            if (!(!wolfe && gn[k] > cfg.ls_grad_tol)) {
              stalled[k] = 0;
              done = true;
            } else if (dqn[k] * alpha * 2 < cfg.tol && cfg.clip) {
              alpha = 0.0;
              stalled[k] = 0;
              done = true;
            } else if (trials[k] >= 2200) {
              done = true;  // stalled: keeps the last trial's step and set
            }
            if (done) {
              ls[k] = 0;
              --n_ls;
              a_fin[k] = alpha * 2;
              fin_pass[k] = pass;
            } else {
              a_cull[k] = alpha;
            }
          }
        }
        for (int k = 0; k < ns; ++k)
          if (act[k] && fin_pass[k] < pass) ++early;
        if (early) {
          // Adopted set: every iterating scene at the step of its accepted trial (the
          // trial culls above covered only the scenes still searching).
          Geo gd = ga;
          gd.alpha_s = sc_alpha.p;
          put_alpha(a_cull);
          cull_set(gd, 2, sets[other]);
        }
        for (int k = 0; k < ns; ++k) {
          st.ls_trials += trials[k];
          sc_ls[k] += trials[k];
          if (stalled[k]) status = ABD_ERR_LS_STALL;
        }
        cur = other;
      }
      for (int k = 0; k < ns; ++k)
        if (act[k]) st.alpha_min = std::min(st.alpha_min, a_fin[k]);
      put_alpha(a_fin);
      launch_q_update_scene(g, q.p, dq.p, sc_alpha.p, s);
      if (!cfg.line_search) launch_project(g, 1, 0.0, s);
      CK(cudaStreamSynchronize(s));
      auto t4 = clk::now();
      st.t_ipc_ms += ms(t0, t1);
      st.t_solver_ms += ms(t1, t2);
      st.t_ccd_ms += ms(t2, t3);
      st.t_ls_ms += ms(t3, t4);
      st.newton_iters++;
      for (int k = 0; k < ns; ++k) {
        if (!act[k]) continue;
        sc_newton[k]++;
        its_f[k]++;
        bool term = sup_dq[k] < cfg.tol || ++iter[k] >= cfg.max_iter;
        if (cfg.max_iter_frame > 0 && its_f[k] >= cfg.max_iter_frame) term = true;
        if (term) {
          act[k] = 0;
          --n_act;
        }
      }
    }
    for (int k = 0; k < ns; ++k) ++iter[k];
    launch_frame_end(q.p, q0.p, dqdt.p, n12, P.dt, s);
    CK(cudaStreamSynchronize(s));
    last_cull_set = cur;
    return status;
  }
};

}  // namespace abd

using abd::Engine;

struct abd_handle {
  Engine e;
};

namespace {
thread_local std::string g_last_error;  // errors of calls without a handle, per host thread

struct ProfScope {
  abd::Prof* prev;
  explicit ProfScope(abd_handle* h) : prev(abd::g_prof) { abd::g_prof = h ? &h->e.prof : nullptr; }
  ~ProfScope() { abd::g_prof = prev; }
};

template <typename F>
int guarded(abd_handle* h, F&& f) {
  ProfScope ps(h);
  try {
    return f();
  } catch (const abd::CudaError& ce) {
    std::string m = std::string(ce.where) + ": " + cudaGetErrorString(ce.code);
    if (h) h->e.err = m;
    g_last_error = m;
    return ABD_ERR_CUDA;
  } catch (const std::invalid_argument& ia) {
    if (h) h->e.err = ia.what();
    g_last_error = ia.what();
    return ABD_ERR_INVALID;
  } catch (const std::exception& ex) {
    if (h) h->e.err = ex.what();
    g_last_error = ex.what();
    return ABD_ERR_CUDA;
  }
}
}  // namespace

extern "C" {

int abd_create(const abd_scene_desc* scene, const abd_config* cfg, abd_handle** out) {
  if (!scene || !cfg || !out || scene->n_bodies <= 0) return ABD_ERR_INVALID;
  abd_handle* h = new abd_handle();
  int rc = guarded(h, [&]() {
    h->e.init(scene, cfg);
    return (int)ABD_OK;
  });
  if (rc != ABD_OK) {
    delete h;
    *out = nullptr;
    return rc;
  }
  *out = h;
  return ABD_OK;
}

void abd_destroy(abd_handle* h) { delete h; }

const char* abd_last_error(abd_handle* h) { return h ? h->e.err.c_str() : g_last_error.c_str(); }

int abd_step(abd_handle* h, double dt, int n_frames, abd_frame_stats* stats) {
  if (!h || n_frames < 0) return ABD_ERR_INVALID;
  return guarded(h, [&]() {
    abd_frame_stats st;
    std::memset(&st, 0, sizeof(st));
    st.toi_min = 1.0;
    st.alpha_min = 1.0;
    if (dt > 0) h->e.P.dt = dt;
    std::fill(h->e.sc_newton.begin(), h->e.sc_newton.end(), 0);
    std::fill(h->e.sc_ls.begin(), h->e.sc_ls.end(), 0);
    std::fill(h->e.sc_pcg.begin(), h->e.sc_pcg.end(), 0);
    long long launches0 = h->e.prof.launches;
    cudaEvent_t ev0, ev1;
    CK(cudaEventCreate(&ev0));
    CK(cudaEventCreate(&ev1));
    CK(cudaEventRecord(ev0, h->e.s));
    int rc = ABD_OK;
    for (int f = 0; f < n_frames; ++f) {
      rc = h->e.step_frame(st);
      st.frames++;
      if (rc != ABD_OK && rc != ABD_ERR_PCG_NOCONV && rc != ABD_ERR_LS_STALL) break;
    }
    st.status = rc;
    CK(cudaEventRecord(ev1, h->e.s));
    CK(cudaEventSynchronize(ev1));
    float dms = 0;
    CK(cudaEventElapsedTime(&dms, ev0, ev1));
    st.device_ms = dms;
    cudaEventDestroy(ev0);
    cudaEventDestroy(ev1);
    h->e.prof.flush();
    st.kernel_launches = h->e.prof.launches - launches0;
    if (stats) *stats = st;
    return rc;
  });
}

int abd_get_state(abd_handle* h, double* q0, double* qdot) {
  if (!h) return ABD_ERR_INVALID;
  return guarded(h, [&]() {
    size_t n = 12 * (size_t)h->e.nb * sizeof(double);
    if (q0) CK(cudaMemcpyAsync(q0, h->e.q0.p, n, cudaMemcpyDeviceToHost, h->e.s));
    if (qdot) CK(cudaMemcpyAsync(qdot, h->e.dqdt.p, n, cudaMemcpyDeviceToHost, h->e.s));
    CK(cudaStreamSynchronize(h->e.s));
    return (int)ABD_OK;
  });
}

int abd_set_state(abd_handle* h, const double* q0, const double* qdot) {
  if (!h) return ABD_ERR_INVALID;
  return guarded(h, [&]() {
    size_t n = 12 * (size_t)h->e.nb * sizeof(double);
    if (q0) {
      CK(cudaMemcpyAsync(h->e.q0.p, q0, n, cudaMemcpyHostToDevice, h->e.s));
      CK(cudaMemcpyAsync(h->e.q.p, q0, n, cudaMemcpyHostToDevice, h->e.s));
    }
    if (qdot) CK(cudaMemcpyAsync(h->e.dqdt.p, qdot, n, cudaMemcpyHostToDevice, h->e.s));
    CK(cudaStreamSynchronize(h->e.s));
    return (int)ABD_OK;
  });
}

int abd_get_counts(abd_handle* h, int* n_bodies, int* n_vertices, int* n_edges, int* n_faces) {
  if (!h) return ABD_ERR_INVALID;
  if (n_bodies) *n_bodies = h->e.nb;
  if (n_vertices) *n_vertices = h->e.nv;
  if (n_edges) *n_edges = h->e.ne;
  if (n_faces) *n_faces = h->e.nf;
  return ABD_OK;
}

int abd_get_iter(abd_handle* h) { return h ? h->e.iter[0] : -1; }

int abd_get_scene_count(abd_handle* h) { return h ? h->e.ns : -1; }

int abd_get_scene_stats(abd_handle* h, int* newton_iters, int* ls_trials, int* pcg_iters, int* iter) {
  if (!h) return ABD_ERR_INVALID;
  for (int k = 0; k < h->e.ns; ++k) {
    if (newton_iters) newton_iters[k] = h->e.sc_newton[k];
    if (ls_trials) ls_trials[k] = h->e.sc_ls[k];
    if (pcg_iters) pcg_iters[k] = h->e.sc_pcg[k];
    if (iter) iter[k] = h->e.iter[k];
  }
  return ABD_OK;
}

int abd_profile(abd_handle* h, int enable) {
  if (!h) return ABD_ERR_INVALID;
  return guarded(h, [&]() {
    h->e.prof.reset();
    h->e.prof.on = enable != 0;
    return (int)ABD_OK;
  });
}

int abd_kernel_times(abd_handle* h, int max_n, char* names, double* total_ms, long long* launches) {
  return abd_kernel_work(h, max_n, names, total_ms, launches, nullptr, nullptr);
}

int abd_kernel_work(abd_handle* h, int max_n, char* names, double* total_ms, long long* launches, double* units,
                    double* bytes) {
  if (!h) return ABD_ERR_INVALID;
  h->e.prof.flush();
  int n = 0;
  for (int t = 0; t < abd::K_NTAGS && n < max_n; ++t) {
    if (names) {
      std::strncpy(names + 32 * n, abd::kTagNames[t], 31);
      names[32 * n + 31] = 0;
    }
    if (total_ms) total_ms[n] = h->e.prof.ms[t];
    if (launches) launches[n] = h->e.prof.cnt[t];
    if (units) units[n] = h->e.prof.units[t];
    if (bytes) bytes[n] = h->e.prof.bytes[t];
    ++n;
  }
  return n;
}
int abd_set_iter(abd_handle* h, int it) {
  if (!h) return ABD_ERR_INVALID;
  for (auto& v : h->e.iter) v = it;
  return ABD_OK;
}

int abd_cull(abd_handle* h, int vtn, const double* q, const double* dq, int* counts, double* toi) {
  if (!h || !q || vtn < 1 || vtn > 3) return ABD_ERR_INVALID;
  return guarded(h, [&]() {
    Engine& e = h->e;
    size_t n = 12 * (size_t)e.nb;
    CK(cudaMemcpyAsync(e.q.p, q, n * sizeof(double), cudaMemcpyHostToDevice, e.s));
    if (dq) CK(cudaMemcpyAsync(e.dq.p, dq, n * sizeof(double), cudaMemcpyHostToDevice, e.s));
    else CK(cudaMemsetAsync(e.dq.p, 0, n * sizeof(double), e.s));
    std::vector<double> tp(e.ns, 1.0), tg(e.ns, 1.0);
    abd::Geo g = e.geo();
    abd::PairSet& S = e.sets[e.cur];
    if (vtn == 3 && e.cfg.iaabb <= 1) {
      std::vector<double> tb(e.ns, 1.0);
      abd::sh_bound(g, e.P, e.sh, S, e.shw, e.cs, tb.data(), e.s);
      double t = 1.0;
      for (int k = 0; k < e.ns; ++k) t = std::min(t, tb[k]);
      if (toi) *toi = t;
      return (int)ABD_OK;
    }
    if (vtn == 3) abd::cull(g, e.P, vtn, 1.0, e.cs, e.sets[2], tp.data(), tg.data(), e.s);
    else e.cull_set(g, vtn == 1 ? 1 : 2, S);
    CK(cudaStreamSynchronize(e.s));
    if (vtn == 3) {
      double t = 1.0;
      for (int k = 0; k < e.ns; ++k) t = std::min(t, e.cfg.ground ? std::min(tp[k], tg[k]) : tp[k]);
      if (toi) *toi = t;
      if (counts) counts[3] = e.sets[2].nov;
    } else {
      e.last_cull_set = e.cur;
      if (counts) {
        counts[0] = S.npt;
        counts[1] = S.nee;
        counts[2] = S.nvg;
        counts[3] = S.nov;
      }
    }
    return (int)ABD_OK;
  });
}

int abd_get_pairs(abd_handle* h, int* pt, int* pt_type, int* ee, int* ee_type, int* vg) {
  if (!h) return ABD_ERR_INVALID;
  return guarded(h, [&]() {
    Engine& e = h->e;
    CK(cudaStreamSynchronize(e.s));
    abd::PairSet& S = e.sets[e.last_cull_set];
    std::vector<int8_t> t8(std::max(S.npt, S.nee) + 1);
    if (pt && S.npt) CK(cudaMemcpy(pt, S.pt.p, 4 * (size_t)S.npt * sizeof(int), cudaMemcpyDeviceToHost));
    if (pt_type && S.npt) {
      CK(cudaMemcpy(t8.data(), S.pt_ty.p, S.npt, cudaMemcpyDeviceToHost));
      for (int i = 0; i < S.npt; ++i) pt_type[i] = t8[i];
    }
    if (ee && S.nee) CK(cudaMemcpy(ee, S.ee.p, 4 * (size_t)S.nee * sizeof(int), cudaMemcpyDeviceToHost));
    if (ee_type && S.nee) {
      CK(cudaMemcpy(t8.data(), S.ee_ty.p, S.nee, cudaMemcpyDeviceToHost));
      for (int i = 0; i < S.nee; ++i) ee_type[i] = t8[i];
    }
    if (vg && S.nvg) CK(cudaMemcpy(vg, S.vg.p, 2 * (size_t)S.nvg * sizeof(int), cudaMemcpyDeviceToHost));
    return (int)ABD_OK;
  });
}

static int newton_system_at(Engine& e, const double* q) {
  size_t n = 12 * (size_t)e.nb;
  CK(cudaMemcpyAsync(e.q.p, q, n * sizeof(double), cudaMemcpyHostToDevice, e.s));
  CK(cudaMemsetAsync(e.dq.p, 0, n * sizeof(double), e.s));
  abd::Geo g = e.geo();
  abd::launch_project(g, 0, 0.0, e.s);
  e.cull_set(g, 1, e.sets[e.cur]);
  abd::assemble(g, e.P, e.sets[e.cur], e.nbufs, e.s);
  CK(cudaStreamSynchronize(e.s));
  e.last_cull_set = e.cur;
  return ABD_OK;
}

int abd_newton_system(abd_handle* h, const double* q, double* grad, double* diag, int* n_off, int* off_keys,
                      double* off_vals, int max_off) {
  if (!h || !q) return ABD_ERR_INVALID;
  return guarded(h, [&]() {
    Engine& e = h->e;
    newton_system_at(e, q);
    abd::PairSet& S = e.sets[e.cur];
    if (grad) CK(cudaMemcpy(grad, e.nbufs.grad.p, 12 * (size_t)e.nb * sizeof(double), cudaMemcpyDeviceToHost));
    if (diag) CK(cudaMemcpy(diag, e.nbufs.D.p, 144 * (size_t)e.nb * sizeof(double), cudaMemcpyDeviceToHost));
    int nov = S.nov;
    std::vector<int> has(nov + 1), oi(nov + 1), oj(nov + 1);
    if (nov) {
      CK(cudaMemcpy(has.data(), e.nbufs.has.p, nov * sizeof(int), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(oi.data(), S.ovI.p, nov * sizeof(int), cudaMemcpyDeviceToHost));
      CK(cudaMemcpy(oj.data(), S.ovJ.p, nov * sizeof(int), cudaMemcpyDeviceToHost));
    }
    int k = 0;
    for (int u = 0; u < nov; ++u) {
      if (!has[u]) continue;
      if (off_keys && k < max_off) {
        off_keys[2 * k] = oi[u];
        off_keys[2 * k + 1] = oj[u];
        CK(cudaMemcpy(off_vals + 144 * (size_t)k, e.nbufs.ovr.p + (size_t)u * abd::CONTRIB + 288,
                      144 * sizeof(double), cudaMemcpyDeviceToHost));
      }
      ++k;
    }
    if (n_off) *n_off = k;
    return (int)ABD_OK;
  });
}

// Line-search energy terms at q + dq with the friction lagged at q: the quantities of the
// first trial of ABD::line_search at alpha = 1 (line_search.cpp:88-110; E_barrier_plus_inert
// energy.cpp:19-86, E_fric :195-258, E_ground :261-270).
int abd_energy(abd_handle* h, const double* q, const double* dq, double* terms, int* counts, double* e_pt,
               double* e_ee, double* e_vg, double* f_pt, double* f_ee, double* f_vg) {
  if (!h || !q || !dq) return ABD_ERR_INVALID;
  return guarded(h, [&]() {
    Engine& e = h->e;
    const int nb = e.nb, ns = e.ns;
    const size_t n = 12 * (size_t)nb;
    newton_system_at(e, q);  // culls at q and assembles there: the lagged friction of that set
    abd::PairSet& L = e.sets[e.cur];
    abd::PairSet& T = e.sets[1 - e.cur];
    CK(cudaMemcpyAsync(e.dq.p, dq, n * sizeof(double), cudaMemcpyHostToDevice, e.s));
    abd::Geo g = e.geo();
    e.cull_set(g, 2, T, 1.0);  // the set at q + dq; positions at q + dq stay in X
    std::vector<double> tot(ns);
    abd::energy(g, e.P, 1.0, T, L, true, e.nbufs, e.s, tot.data());
    const int c[6] = {T.npt, T.nee, T.nvg, L.npt, L.nee, L.nvg};
    size_t m = nb;
    for (int k = 0; k < 6; ++k) m += c[k];
    abd::DBuf<double> d_out;
    d_out.ensure(m + 1);
    abd::energy_terms(g, e.P, 1.0, T, L, d_out.p, e.s);
    std::vector<double> v(m);
    CK(cudaMemcpyAsync(v.data(), d_out.p, m * sizeof(double), cudaMemcpyDeviceToHost, e.s));
    // scene of each listed pair: the scene of its first body
    std::vector<int> lists[6];
    const abd::PairSet* src[6] = {&T, &T, &T, &L, &L, &L};
    for (int k = 0; k < 6; ++k) {
      const int stride = (k % 3 == 2) ? 2 : 4;
      const int* d = (k % 3 == 0) ? src[k]->pt.p : (k % 3 == 1) ? src[k]->ee.p : src[k]->vg.p;
      lists[k].resize((size_t)stride * c[k]);
      if (c[k]) CK(cudaMemcpyAsync(lists[k].data(), d, lists[k].size() * sizeof(int), cudaMemcpyDeviceToHost, e.s));
    }
    CK(cudaStreamSynchronize(e.s));
    d_out.release();
    std::vector<int> bsc(nb);
    for (int k = 0; k < ns; ++k)
      for (int b = e.h_sc_beg[k]; b < e.h_sc_end[k]; ++b) bsc[b] = k;
    // terms per scene: inertia + orthogonality, PT, EE, ground barrier, friction, and the
    // total as the line search sums it
    if (terms) {
      for (int k = 0; k < 6 * ns; ++k) terms[k] = 0.0;
      for (int b = 0; b < nb; ++b) terms[6 * bsc[b]] += v[b];
      size_t o = nb;
      for (int k = 0; k < 6; ++k) {
        const int stride = (k % 3 == 2) ? 2 : 4;
        const int slot = k < 3 ? 1 + k : 4;
        for (int i = 0; i < c[k]; ++i) terms[6 * bsc[lists[k][(size_t)stride * i]] + slot] += v[o + i];
        o += c[k];
      }
      for (int k = 0; k < ns; ++k) terms[6 * k + 5] = tot[k];
    }
    double* outs[6] = {e_pt, e_ee, e_vg, f_pt, f_ee, f_vg};
    size_t o = nb;
    for (int k = 0; k < 6; ++k) {
      if (outs[k]) std::memcpy(outs[k], v.data() + o, c[k] * sizeof(double));
      o += c[k];
    }
    if (counts)
      for (int k = 0; k < 6; ++k) counts[k] = c[k];
    e.last_cull_set = 1 - e.cur;
    return (int)ABD_OK;
  });
}

int abd_set_friction(abd_handle* h, double mu) {
  if (!h || !(mu >= 0.0)) return ABD_ERR_INVALID;
  h->e.P.mu = mu;
  h->e.cfg.mu = mu;
  return ABD_OK;
}

int abd_set_trace(abd_handle* h, const char* folder, int ts, int starting_ts, int ending_ts, const char* config_json,
                  const char* scene_json) {
  if (!h || ts < 0) return ABD_ERR_INVALID;
  Engine& e = h->e;
  if (folder) e.trace_folder = folder;
  e.ts = ts;
  e.starting_ts = starting_ts;
  e.ending_ts = ending_ts;
  if (config_json) e.trace_config = config_json;
  if (scene_json) e.trace_scene = scene_json;
  return ABD_OK;
}

int abd_get_trace(abd_handle* h, int* ts, int* starting_ts, int* ending_ts, char* folder, int folder_cap) {
  if (!h) return ABD_ERR_INVALID;
  Engine& e = h->e;
  if (ts) *ts = e.ts;
  if (starting_ts) *starting_ts = e.starting_ts;
  if (ending_ts) *ending_ts = e.ending_ts;
  if (folder && folder_cap > 0) {
    std::strncpy(folder, e.trace_folder.c_str(), folder_cap - 1);
    folder[folder_cap - 1] = 0;
  }
  if (folder && folder_cap > 0 && (int)e.trace_folder.size() >= folder_cap) return ABD_ERR_INVALID;
  return ABD_OK;
}

int abd_trace_files(abd_handle* h, const char** config_json, const char** scene_json) {
  if (!h) return ABD_ERR_INVALID;
  if (config_json) *config_json = h->e.trace_config.empty() ? nullptr : h->e.trace_config.c_str();
  if (scene_json) *scene_json = h->e.trace_scene.empty() ? nullptr : h->e.trace_scene.c_str();
  return ABD_OK;
}

int abd_autotune_info(abd_handle* h, int* steps, double* ms) {
  if (!h) return ABD_ERR_INVALID;
  const abd::CullScratch& cs = h->e.cs;
  for (int m = 0; m < 2; ++m) {
    if (steps) steps[m] = cs.narrow_variant[m] >= 0 ? abd::narrow_step_of(m ? 2 : 0, cs.narrow_variant[m]) : 0;
    if (ms)
      for (int v = 0; v < 3; ++v) ms[3 * m + v] = cs.narrow_ms[m][v];
  }
  return ABD_OK;
}

int abd_adjoint_stats(abd_handle* h, int* iterations, double* rel_residual) {
  if (!h) return ABD_ERR_INVALID;
  if (iterations) *iterations = h->e.adj_iters;
  if (rel_residual) *rel_residual = h->e.adj_residual;
  return ABD_OK;
}

int abd_get_friction(abd_handle* h, double* mu) {
  if (!h || !mu) return ABD_ERR_INVALID;
  *mu = h->e.P.mu;
  return ABD_OK;
}

// Adjoint of one converged frame by implicit differentiation. At the frame's solution
// q_{t+1} the gradient r(q; q_t, v_t, mu) of the incremental potential vanishes, so
// dL/dtheta = -w^T dr/dtheta with J^T w = dL/dq_{t+1}, J the Jacobian of r at q_{t+1}:
//   J = H + C + F,
// H the exact Hessian (no PSD projection, no damping, the ground barrier's full second
// derivative, the friction Hessian with every tangent frame and multiplier held), C the
// coupling through the ground-friction multipliers (which follow the vertex heights), F
// the point-triangle / edge-edge friction forces' Jacobian through their tangent frames,
// closest points and multipliers (all recomputed at every Newton iterate by the reference,
// pt_ipc.cpp:22-107, ee_ipc.cpp:21-118). J is not symmetric (the friction force is not a
// potential's gradient once its frame moves) and H can be indefinite, so J^T w = g is
// solved by flexible GMRES preconditioned with the Newton matrix of the forward step at
// q_{t+1} (PSD-projected, SPD), applied by the block-Jacobi PCG. Then
// dr/dq_t = -M - mu K (inertia through q_tilde, friction through the reference positions
// x(q_t), K the friction Hessian with frames held), dr/dv_t = -dt M, dr/dmu =
// r_friction / mu; K and r_friction are assembled at mu = 1.
int abd_adjoint_frame(abd_handle* h, const double* q_t, const double* v_t, const double* q_next,
                      const double* gq_next, double* gq_t, double* gv_t, double* gmu) {
  if (!h || !q_t || !v_t || !q_next || !gq_next || !gq_t || !gv_t) return ABD_ERR_INVALID;
  return guarded(h, [&]() {
    Engine& e = h->e;
    const int nb = e.nb;
    const int n = 12 * nb;
    abd::NewtonBufs& B = e.nbufs;
    cudaStream_t s = e.s;
    CK(cudaMemcpyAsync(e.q0.p, q_t, n * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(e.dqdt.p, v_t, n * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemcpyAsync(e.q.p, q_next, n * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(e.dq.p, 0, n * sizeof(double), s));
    abd::Geo g = e.geo();
    abd::PairSet& S = e.sets[e.cur];
    abd::launch_project(g, 0, 0.0, s);  // reference positions x(q_t)
    e.cull_set(g, 1, S);                // positions x(q_{t+1}) and their pair set
    // J's exact part, kept aside, and the frame Jacobians of the friction forces
    abd::Params Pe = e.P;
    Pe.psd = 0;
    Pe.damp = 0;
    Pe.exact = 1;
    Pe.terms = abd::TERM_ALL;
    abd::assemble(g, Pe, S, B, s);
    const int nov = S.nov;
    B.D_ex.ensure(144 * (size_t)nb);
    B.ovr_ex.ensure((size_t)abd::CONTRIB * nov + 1);
    B.has_ex.ensure(nov + 1);
    CK(cudaMemcpyAsync(B.D_ex.p, B.D.p, 144 * (size_t)nb * sizeof(double), cudaMemcpyDeviceToDevice, s));
    if (nov) {
      CK(cudaMemcpyAsync(B.ovr_ex.p, B.ovr.p, (size_t)abd::CONTRIB * nov * sizeof(double), cudaMemcpyDeviceToDevice,
                         s));
      CK(cudaMemcpyAsync(B.has_ex.p, B.has.p, nov * sizeof(int), cudaMemcpyDeviceToDevice, s));
    }
    abd::fric_frame_jacobians(g, Pe, S, B, s);
    const bool vg_coupling = e.P.mu > 0.0 && e.cfg.ground && e.cfg.vg_fric && S.nvg > 0;
    // the preconditioner: the forward step's (projected, undamped) Newton matrix
    abd::Params Pp = e.P;
    Pp.psd = 1;
    Pp.damp = 0;
    Pp.exact = 0;
    Pp.terms = abd::TERM_ALL;
    abd::assemble(g, Pp, S, B, s);
    e.put_on(std::vector<char>(e.ns, 1));
    abd::SolveOpts po = e.solve_opts();
    po.rel_tol = 1e-10;
    po.refine = 0;
    po.dense = 0;
    const std::vector<char> all_on(e.ns, 1);
    const int m = 40, max_restarts = 12;
    B.adj_V.ensure((size_t)(m + 1) * n);
    B.adj_Z.ensure((size_t)m * n);
    B.adj_w.ensure(n);
    B.adj_t.ensure(n);
    B.adj_x.ensure(n);
    double* V = B.adj_V.p;
    double* Z = B.adj_Z.p;
    double* wv = B.adj_w.p;
    double* tv = B.adj_t.p;
    double* xv = B.adj_x.p;
    int st = ABD_OK;
    // out = J^T z
    auto apply = [&](const double* z, double* out) {
      abd::spmv_blocks(g, S, B.has_ex.p, B.ovr_ex.p, B.D_ex.p, z, out, s);
      if (vg_coupling) {
        abd::vg_lag_adjoint(g, Pe, S, z, tv, s);
        abd::dev_axpby(n, 1.0, tv, 1.0, out, s);
      }
      abd::fric_frame_apply_t(g, S, B, z, tv, s);
      abd::dev_axpby(n, 1.0, tv, 1.0, out, s);
    };
    // z = P^-1 v by the PCG on the preconditioner's system
    auto precond = [&](const double* v, double* z) {
      CK(cudaMemcpyAsync(B.grad.p, v, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
      int ps = 0;
      abd::pcg_solve(g, S, B, po, e.sc_on.p, all_on, e.dq.p, s, &ps, nullptr);
      if (ps == ABD_ERR_NOT_SPD) st = ABD_ERR_NOT_SPD;
      CK(cudaMemcpyAsync(z, B.x.p, n * sizeof(double), cudaMemcpyDeviceToDevice, s));
    };
    CK(cudaMemcpyAsync(V, gq_next, n * sizeof(double), cudaMemcpyHostToDevice, s));
    CK(cudaMemsetAsync(xv, 0, n * sizeof(double), s));
    const double bnorm = std::sqrt(abd::dev_dot(n, V, V, B, s));
    const double tol = 1e-12 * bnorm;
    double beta = bnorm;
    bool converged = bnorm == 0.0;
    std::vector<double> H((size_t)(m + 1) * m), cs(m), sn(m), gg(m + 1), y(m);
    int total_its = 0;
    double last_res = bnorm;
    for (int rs = 0; rs < max_restarts && !converged && st == ABD_OK; ++rs) {
      if (rs > 0) {  // restart from the true residual b - J^T x
        apply(xv, wv);
        CK(cudaMemcpyAsync(V, gq_next, n * sizeof(double), cudaMemcpyHostToDevice, s));
        abd::dev_axpby(n, -1.0, wv, 1.0, V, s);
        beta = std::sqrt(abd::dev_dot(n, V, V, B, s));
        if (beta <= tol) {
          converged = true;
          break;
        }
      }
      abd::dev_axpby(n, 0.0, V, 1.0 / beta, V, s);
      std::fill(gg.begin(), gg.end(), 0.0);
      gg[0] = beta;
      int k = 0;
      for (; k < m; ++k) {
        double* vk = V + (size_t)k * n;
        double* zk = Z + (size_t)k * n;
        double* vn = V + (size_t)(k + 1) * n;
        precond(vk, zk);
        apply(zk, vn);
        for (int i = 0; i <= k; ++i) {  // modified Gram-Schmidt
          const double hik = abd::dev_dot(n, vn, V + (size_t)i * n, B, s);
          H[(size_t)i * m + k] = hik;
          abd::dev_axpby(n, -hik, V + (size_t)i * n, 1.0, vn, s);
        }
        const double hn = std::sqrt(abd::dev_dot(n, vn, vn, B, s));
        H[(size_t)(k + 1) * m + k] = hn;
        if (hn > 0.0) abd::dev_axpby(n, 0.0, vn, 1.0 / hn, vn, s);
        for (int i = 0; i < k; ++i) {  // the earlier rotations on the new column
          const double a0 = H[(size_t)i * m + k], a1 = H[(size_t)(i + 1) * m + k];
          H[(size_t)i * m + k] = cs[i] * a0 + sn[i] * a1;
          H[(size_t)(i + 1) * m + k] = -sn[i] * a0 + cs[i] * a1;
        }
        const double a0 = H[(size_t)k * m + k], a1 = H[(size_t)(k + 1) * m + k];
        const double rr = std::hypot(a0, a1);
        cs[k] = rr > 0.0 ? a0 / rr : 1.0;
        sn[k] = rr > 0.0 ? a1 / rr : 0.0;
        H[(size_t)k * m + k] = rr;
        H[(size_t)(k + 1) * m + k] = 0.0;
        gg[k + 1] = -sn[k] * gg[k];
        gg[k] = cs[k] * gg[k];
        ++total_its;
        last_res = std::fabs(gg[k + 1]);
        if (std::fabs(gg[k + 1]) <= tol || hn == 0.0) {
          ++k;
          converged = true;
          break;
        }
      }
      // x += Z y with H y = g (upper triangular, k x k)
      for (int i = k - 1; i >= 0; --i) {
        double v = gg[i];
        for (int j = i + 1; j < k; ++j) v -= H[(size_t)i * m + j] * y[j];
        y[i] = v / H[(size_t)i * m + i];
      }
      for (int i = 0; i < k; ++i) abd::dev_axpby(n, y[i], Z + (size_t)i * n, 1.0, xv, s);
    }
    e.adj_iters = total_its;
    e.adj_residual = bnorm > 0.0 ? last_res / bnorm : 0.0;
    if (st != ABD_OK) return st;
    if (!converged) st = ABD_ERR_PCG_NOCONV;
    std::vector<double> w(n), yk(n), gf(n), mass(nb), Ic(nb);
    CK(cudaMemcpyAsync(w.data(), xv, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    // friction terms alone at mu = 1, frames held: K w and r_friction / mu
    abd::Params Pf = Pe;
    Pf.terms = abd::TERM_FRICTION;
    Pf.mu = 1.0;
    abd::assemble(g, Pf, S, B, s);
    abd::spmv(g, S, B, xv, B.r.p, s);
    CK(cudaMemcpyAsync(yk.data(), B.r.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(gf.data(), B.grad.p, n * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(mass.data(), e.mass.p, nb * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaMemcpyAsync(Ic.data(), e.Ic.p, nb * sizeof(double), cudaMemcpyDeviceToHost, s));
    CK(cudaStreamSynchronize(s));
    double gm = 0.0, mu = e.P.mu, dt = e.P.dt;
    for (int b = 0; b < nb; ++b)
      for (int i = 0; i < 12; ++i) {
        size_t k = 12 * (size_t)b + i;
        if (mass[b] < 0.0) {  // static: q_{t+1} = q_t
          gq_t[k] = gq_next[k];
          gv_t[k] = 0.0;
          continue;
        }
        double mi = i < 3 ? mass[b] : Ic[b];
        gq_t[k] = mi * w[k] + mu * yk[k];
        gv_t[k] = dt * mi * w[k];
        gm -= gf[k] * w[k];
      }
    if (gmu) *gmu = gm;
    return st;
  });
}

int abd_newton_dq(abd_handle* h, const double* q, double* dq, int* pcg_iters) {
  if (!h || !q || !dq) return ABD_ERR_INVALID;
  return guarded(h, [&]() {
    Engine& e = h->e;
    newton_system_at(e, q);
    int st = 0;
    e.put_on(std::vector<char>(e.ns, 1));
    int its = abd::pcg_solve(e.geo(), e.sets[e.cur], e.nbufs, e.solve_opts(), e.sc_on.p, std::vector<char>(e.ns, 1),
                             e.dq.p, e.s, &st, nullptr);
    if (pcg_iters) *pcg_iters = its;
    CK(cudaMemcpy(dq, e.dq.p, 12 * (size_t)e.nb * sizeof(double), cudaMemcpyDeviceToHost));
    return st;
  });
}

}  // extern "C"
