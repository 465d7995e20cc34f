// File front end of the C ABI: reads the reference's config.json
// (view/control.cpp:19-111) and scene JSON (test_cases/spinning_cube.cpp:56-127) with a
// small JSON reader, loads Wavefront OBJ meshes (the reference loads them through
// assimp, view/model.h) and builds the scene descriptor for abd_create.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <filesystem>
#include <fstream>
#include <map>
#include <memory>
#include <set>
#include <sstream>
#include <string>
#include <vector>

#include "../../include/abd_gb300.h"

namespace {

struct JV {
  enum T { NUL, BOOL, NUM, STR, ARR, OBJ } t = NUL;
  bool b = false;
  double n = 0;
  std::string s;
  std::vector<JV> a;
  std::vector<std::pair<std::string, JV>> o;
  const JV* get(const std::string& k) const {
    for (auto& kv : o)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
  double num(const std::string& k, double def) const {
    const JV* v = get(k);
    if (!v) return def;
    if (v->t == NUM) return v->n;
    if (v->t == BOOL) return v->b ? 1.0 : 0.0;
    return def;
  }
  bool flag(const std::string& k, bool def) const {
    const JV* v = get(k);
    if (!v) return def;
    if (v->t == BOOL) return v->b;
    if (v->t == NUM) return v->n != 0;
    return def;
  }
};

struct Parser {
  const char* p;
  const char* end;
  bool ok = true;
  void ws() {
    while (p < end && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
  }
  JV parse() {
    ws();
    JV v;
    if (p >= end) { ok = false; return v; }
    if (*p == '{') {
      ++p;
      v.t = JV::OBJ;
      ws();
      if (p < end && *p == '}') { ++p; return v; }
      while (ok) {
        ws();
        JV k = parse();
        if (k.t != JV::STR) { ok = false; break; }
        ws();
        if (p >= end || *p != ':') { ok = false; break; }
        ++p;
        JV val = parse();
        v.o.emplace_back(k.s, val);
        ws();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == '}') { ++p; break; }
        ok = false;
      }
    } else if (*p == '[') {
      ++p;
      v.t = JV::ARR;
      ws();
      if (p < end && *p == ']') { ++p; return v; }
      while (ok) {
        v.a.push_back(parse());
        ws();
        if (p < end && *p == ',') { ++p; continue; }
        if (p < end && *p == ']') { ++p; break; }
        ok = false;
      }
    } else if (*p == '"') {
      ++p;
      v.t = JV::STR;
      while (p < end && *p != '"') {
        if (*p == '\\' && p + 1 < end) ++p;
        v.s.push_back(*p++);
      }
      if (p < end) ++p;
    } else if (!strncmp(p, "true", 4)) {
      v.t = JV::BOOL; v.b = true; p += 4;
    } else if (!strncmp(p, "false", 5)) {
      v.t = JV::BOOL; v.b = false; p += 5;
    } else if (!strncmp(p, "null", 4)) {
      p += 4;
    } else {
      char* e;
      v.t = JV::NUM;
      v.n = strtod(p, &e);
      if (e == p) ok = false;
      p = e;
    }
    return v;
  }
};

bool read_file(const std::string& path, std::string& out) {
  std::ifstream f(path, std::ios::binary);
  if (!f) return false;
  std::stringstream ss;
  ss << f.rdbuf();
  out = ss.str();
  return true;
}

bool parse_json(const std::string& path, JV& out) {
  std::string txt;
  if (!read_file(path, txt)) return false;
  Parser ps{txt.data(), txt.data() + txt.size()};
  out = ps.parse();
  return ps.ok;
}

struct Mesh {
  std::vector<double> v;
  std::vector<int> f, e;
};

void extract_edges(Mesh& m) {
  std::set<std::pair<int, int>> s;
  for (size_t i = 0; i + 2 < m.f.size(); i += 3) {
    int a = m.f[i], b = m.f[i + 1], c = m.f[i + 2];
    int pr[3][2] = {{a, b}, {b, c}, {a, c}};
    for (auto& q : pr) s.insert({std::min(q[0], q[1]), std::max(q[0], q[1])});
  }
  for (auto& q : s) {
    m.e.push_back(q.first);
    m.e.push_back(q.second);
  }
}

bool read_obj(const std::string& path, Mesh& m) {
  std::ifstream f(path);
  if (!f) return false;
  std::string line;
  while (std::getline(f, line)) {
    std::istringstream ls(line);
    std::string tag;
    ls >> tag;
    if (tag == "v") {
      double x, y, z;
      ls >> x >> y >> z;
      m.v.push_back(x); m.v.push_back(y); m.v.push_back(z);
    } else if (tag == "f") {
      std::vector<int> idx;
      std::string tok;
      while (ls >> tok) idx.push_back(std::atoi(tok.c_str()) - 1);
      for (size_t k = 1; k + 1 < idx.size(); ++k) {
        m.f.push_back(idx[0]); m.f.push_back(idx[k]); m.f.push_back(idx[k + 1]);
      }
    }
  }
  extract_edges(m);
  return true;
}

// model/cube.h:4-70
Mesh cube_mesh() {
  Mesh m;
  const double v[8][3] = {{-0.5, -0.5, -0.5}, {-0.5, -0.5, 0.5}, {-0.5, 0.5, -0.5}, {-0.5, 0.5, 0.5},
                          {0.5, -0.5, -0.5},  {0.5, -0.5, 0.5},  {0.5, 0.5, -0.5},  {0.5, 0.5, 0.5}};
  for (auto& p : v) m.v.insert(m.v.end(), p, p + 3);
  const int q[24] = {0, 1, 3, 2, 4, 5, 1, 0, 4, 0, 2, 6, 2, 3, 7, 6, 1, 5, 7, 3, 5, 4, 6, 7};
  for (int i = 0; i < 6; ++i) {
    const int* f = q + 4 * i;
    int t[6] = {f[0], f[1], f[2], f[2], f[3], f[0]};
    m.f.insert(m.f.end(), t, t + 6);
  }
  for (int i = 0; i < 3; ++i) {
    int di = 1 << (2 - i);
    for (int j = 0; j < 4; ++j) {
      int e0 = q[i * 4 + j];
      m.e.push_back(e0);
      m.e.push_back(e0 + di);
    }
  }
  return m;
}

// Frame file <folder>/<ts> of a trace: 24 doubles per body (player_load, mutils.cpp:257-276).
int read_trace_frame(const std::string& folder, int ts, std::vector<double>& buf) {
  std::ifstream in(folder + "/" + std::to_string(ts), std::ios::binary | std::ios::ate);
  if (!in) return ABD_ERR_IO;
  std::streamsize n = in.tellg();
  if (n != (std::streamsize)(buf.size() * sizeof(double))) return ABD_ERR_IO;
  in.seekg(0);
  in.read(reinterpret_cast<char*>(buf.data()), n);
  return in ? ABD_OK : ABD_ERR_IO;
}

// geometry.cpp:248-264: Rz(a) Ry(b) Rx(c)
void rotation(double a, double b, double c, double R[3][3]) {
  double s1 = std::sin(a), s2 = std::sin(b), s3 = std::sin(c);
  double c1 = std::cos(a), c2 = std::cos(b), c3 = std::cos(c);
  double M[3][3] = {{c1 * c2, c1 * s2 * s3 - c3 * s1, s1 * s3 + c1 * c3 * s2},
                    {c2 * s1, c1 * c3 + s1 * s2 * s3, c3 * s1 * s2 - c1 * s3},
                    {-s2, c2 * s3, c2 * c3}};
  std::memcpy(R, M, sizeof(M));
}

}  // namespace

extern "C" int abd_create_from_files(const char* config_json, const char* scene_json, abd_handle** out) {
  if (!config_json || !scene_json || !out) return ABD_ERR_INVALID;
  JV cfgj, scj;
  if (!parse_json(config_json, cfgj) || cfgj.t != JV::OBJ) return ABD_ERR_IO;
  if (!parse_json(scene_json, scj) || scj.t != JV::ARR) return ABD_ERR_IO;
  abd_config c;
  std::memset(&c, 0, sizeof(c));
  const JV* pd = cfgj.get("params_double");
  const JV* pi = cfgj.get("params_int");
  c.dt = cfgj.num("dt", 1e-2);
  c.kappa = cfgj.num("kappa", 1e-4);
  c.dhat = cfgj.num("dhat", 1e-4);
  c.ortho_kappa = cfgj.num("ortho_kappa", 1e9);
  c.ground_offset = cfgj.get("ground_y") ? -cfgj.num("ground_y", -0.5) : 0.5;
  c.mu = cfgj.num("mu", 0.0);
  c.evh = cfgj.num("evh", 1e-3);
  c.eps_x = cfgj.num("eps_x", 1e-3);
  c.backoff = cfgj.num("backoff", 0.8);
  c.c1 = pd ? pd->num("c1", 1e-4) : 1e-4;
  c.tol = pd ? pd->num("tol", 1e-2) : 1e-2;
  c.max_uk = pd ? pd->num("max_uk", 0.0) : 0.0;
  c.gravity_y = cfgj.flag("gravity", true) ? -9.8 : 0.0;
  c.ls_grad_tol = 1e-3;
  c.pcg_rel_tol = cfgj.num("pcg_rel_tol", 1e-11);
  c.max_iter = (int)cfgj.num("max_iter", 1000);
  c.max_iter_frame = (int)cfgj.num("max_iter_frame", 0);
  c.autotune = cfgj.flag("autotune", true);
  c.tri_direct = cfgj.flag("tri_direct", true);
  c.ground = cfgj.flag("ground", true);
  c.pt = cfgj.flag("pt", true);
  c.ee = cfgj.flag("ee", true);
  c.psd = cfgj.flag("psd", true);
  c.line_search = cfgj.flag("line_search", true);
  c.upper_bound = cfgj.get("uppper_bound") ? cfgj.flag("uppper_bound", true) : cfgj.flag("upper_bound", true);
  c.vg_fric = cfgj.flag("vg_friction", true);
  c.pt_fric = cfgj.flag("pt_friction", true);
  c.ee_fric = cfgj.flag("ee_friction", true);
  c.clip = pi ? (int)pi->num("clip", 0) : 0;
  c.pcg_max_iter = (int)cfgj.num("pcg_max_iter", 5000);
  c.pcg_refine = (int)cfgj.num("pcg_refine", 0);
  c.pcg_refine_tol = cfgj.num("pcg_refine_tol", 1e-8);
  const JV* sv = cfgj.get("solver");
  c.solver = (sv && sv->t == JV::STR && sv->s == "dense") ? 1 : 0;
  c.iaabb = (int)cfgj.num("iaabb", 3);
  c.full_ccd = cfgj.flag("full_ccd", true);
  c.safe_factor = cfgj.num("safe_factor", 1.0);
  const JV* sh = cfgj.get("spatial hashing");
  c.sh_min_xyz = sh ? sh->num("min_xyz", -10.0) : -10.0;
  c.sh_dx = sh ? sh->num("dx", 0.8) : 0.8;
  c.sh_xyz_bits = sh ? (int)sh->num("xyz_bits", 6) : 6;
  c.sh_fix_edge_trajectory = cfgj.flag("sh_fix_edge_trajectory", false);
  c.dq_tol = pd ? pd->num("dq_tol", 0.0) : 0.0;
  const JV* dmp = cfgj.get("damping");
  c.damping = dmp ? dmp->flag("enable", false) : 0;
  c.damp_alpha = dmp ? dmp->num("alpha", 5e-2) : 5e-2;
  c.damp_beta = dmp ? dmp->num("beta", 2.5e-2) : 2.5e-2;

  std::string dir = scene_json;
  size_t sl = dir.find_last_of('/');
  dir = (sl == std::string::npos) ? std::string(".") : dir.substr(0, sl);
  std::map<std::string, std::shared_ptr<Mesh>> cache;
  std::vector<double> q0, qd, mass, Ic, rest;
  std::vector<int> vo{0}, eo{0}, fo{0}, edges, faces;
  for (const JV& it : scj.a) {
    std::shared_ptr<Mesh> mp;
    const JV* obj = it.get("obj");
    if (obj && obj->t == JV::STR) {
      std::string fn = obj->s[0] == '/' ? obj->s : dir + "/" + obj->s;
      auto f = cache.find(fn);
      if (f == cache.end()) {
        auto m = std::make_shared<Mesh>();
        if (!read_obj(fn, *m)) return ABD_ERR_IO;
        cache[fn] = m;
        mp = m;
      } else {
        mp = f->second;
      }
    } else {
      mp = std::make_shared<Mesh>(cube_mesh());
    }
    double om[3] = {0.0, 0.0, 20.0};
    if (const JV* o = it.get("omega"))
      for (int k = 0; k < 3 && k < (int)o->a.size(); ++k) om[k] = o->a[k].n;
    double p[3] = {0, 0, 0}, pdot[3] = {0, 0, 0};
    if (const JV* o = it.get("p"))
      for (int k = 0; k < 3 && k < (int)o->a.size(); ++k) p[k] = o->a[k].n;
    if (const JV* o = it.get("p_dot"))
      for (int k = 0; k < 3 && k < (int)o->a.size(); ++k) pdot[k] = o->a[k].n;
    double R[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
    const double pi_ = 3.14159265358979323846;
    if (const JV* eu = it.get("euler")) {
      rotation(eu->a[2].n / 180.0 * pi_, eu->a[1].n / 180.0 * pi_, eu->a[0].n / 180.0 * pi_, R);
    } else {
      double th = it.num("theta", 0.0) / 180.0 * pi_;
      double s = std::sin(th), cth = std::cos(th);
      R[0][0] = cth; R[1][1] = cth; R[0][1] = -s; R[1][0] = s;
    }
    double m = 1000.0, ic = 1000.0 / 12.0;
    if (it.get("mass")) {
      m = it.num("mass", 1000.0);
      ic = m / 12;
    }
    double qq[12] = {p[0], p[1], p[2]};
    for (int k = 0; k < 3; ++k)
      for (int r = 0; r < 3; ++r) qq[3 + 3 * k + r] = R[r][k];
    // geometry.h:28-35 skew(omega)
    double dq_[12] = {pdot[0], pdot[1], pdot[2], 0, om[2], -om[1], -om[2], 0, om[0], om[1], -om[0], 0};
    q0.insert(q0.end(), qq, qq + 12);
    qd.insert(qd.end(), dq_, dq_ + 12);
    mass.push_back(m);
    Ic.push_back(ic);
    rest.insert(rest.end(), mp->v.begin(), mp->v.end());
    edges.insert(edges.end(), mp->e.begin(), mp->e.end());
    faces.insert(faces.end(), mp->f.begin(), mp->f.end());
    vo.push_back(vo.back() + (int)mp->v.size() / 3);
    eo.push_back(eo.back() + (int)mp->e.size() / 2);
    fo.push_back(fo.back() + (int)mp->f.size() / 3);
  }
  if (mass.empty()) return ABD_ERR_INVALID;
  abd_scene_desc d;
  d.n_bodies = (int)mass.size();
  d.q0 = q0.data();
  d.dqdt = qd.data();
  d.mass = mass.data();
  d.Ic = Ic.data();
  d.vert_off = vo.data();
  d.rest_vertices = rest.data();
  d.edge_off = eo.data();
  d.edges = edges.data();
  d.face_off = fo.data();
  d.faces = faces.data();
  d.scene_id = nullptr;
  // trace settings (view/control.cpp:41, 84-90): a non-negative starting_ts resumes from
  // frame file <trace_folder>/<starting_ts> of a reference trace
  const JV* tf = cfgj.get("trace_folder");
  std::string folder = (tf && tf->t == JV::STR) ? tf->s : std::string("trace");
  int starting_ts = (int)cfgj.num("starting_ts", -1);
  int ending_ts = (int)cfgj.num("ending_ts", 0);
  if (starting_ts >= 0) {
    std::vector<double> buf(24 * (size_t)d.n_bodies);
    if (read_trace_frame(folder, starting_ts, buf) != ABD_OK) return ABD_ERR_IO;
    for (int b = 0; b < d.n_bodies; ++b)
      for (int k = 0; k < 12; ++k) {
        q0[12 * (size_t)b + k] = buf[24 * (size_t)b + k];
        qd[12 * (size_t)b + k] = buf[24 * (size_t)b + 12 + k];
      }
  }
  int rc = abd_create(&d, &c, out);
  if (rc != ABD_OK) return rc;
  abd_set_trace(*out, folder.c_str(), starting_ts >= 0 ? starting_ts : 0, starting_ts, ending_ts, config_json,
                scene_json);
  return ABD_OK;
}

// ---- traces in the reference's binary layout (player_save / player_load,
//      model/mutils.cpp:257-276, 293-329): one file per frame, <folder>/<ts>, holding per
//      body q0 (p, a1, a2, a3) then dqdt as raw doubles ----

extern "C" int abd_trace_save(abd_handle* h, const char* folder, int ts, int init) {
  if (!h || !folder || ts < 0) return ABD_ERR_INVALID;
  int nb = 0;
  abd_get_counts(h, &nb, nullptr, nullptr, nullptr);
  std::vector<double> q0(12 * (size_t)nb), qd(12 * (size_t)nb), buf(24 * (size_t)nb);
  int rc = abd_get_state(h, q0.data(), qd.data());
  if (rc != ABD_OK) return rc;
  namespace fs = std::filesystem;
  std::error_code ec;
  if (init) {  // a new trace: the folder is recreated and the run's config and scene copied in
    fs::remove_all(folder, ec);
    fs::create_directories(folder, ec);
    if (ec) return ABD_ERR_IO;
    const char *cj = nullptr, *sj = nullptr;
    abd_trace_files(h, &cj, &sj);
    for (const char* f : {cj, sj})
      if (f) {
        fs::copy_file(f, fs::path(folder) / fs::path(f).filename(), fs::copy_options::overwrite_existing, ec);
        if (ec) return ABD_ERR_IO;
      }
  } else {
    fs::create_directories(folder, ec);
  }
  for (int b = 0; b < nb; ++b)
    for (int k = 0; k < 12; ++k) {
      buf[24 * (size_t)b + k] = q0[12 * (size_t)b + k];
      buf[24 * (size_t)b + 12 + k] = qd[12 * (size_t)b + k];
    }
  std::ofstream out(std::string(folder) + "/" + std::to_string(ts), std::ios::binary | std::ios::trunc);
  if (!out) return ABD_ERR_IO;
  out.write(reinterpret_cast<const char*>(buf.data()), buf.size() * sizeof(double));
  return out ? ABD_OK : ABD_ERR_IO;
}

extern "C" int abd_trace_load(abd_handle* h, const char* folder, int ts) {
  if (!h || !folder || ts < 0) return ABD_ERR_INVALID;
  int nb = 0;
  abd_get_counts(h, &nb, nullptr, nullptr, nullptr);
  std::vector<double> buf(24 * (size_t)nb), q0(12 * (size_t)nb), qd(12 * (size_t)nb);
  int rc = read_trace_frame(folder, ts, buf);
  if (rc != ABD_OK) return rc;
  for (int b = 0; b < nb; ++b)
    for (int k = 0; k < 12; ++k) {
      q0[12 * (size_t)b + k] = buf[24 * (size_t)b + k];
      qd[12 * (size_t)b + k] = buf[24 * (size_t)b + 12 + k];
    }
  return abd_set_state(h, q0.data(), qd.data());
}

// The reference's viewer loop without its rendering (view/model_view.cpp:282-295): one
// frame per pass; the frame counter advances inside the step (abd.cpp:116) and, when
// recording, the new state is written as frame file <folder>/<ts> (the folder is
// recreated on the pass that starts at ts 0); stops once ts reaches ending_ts.
extern "C" int abd_run(abd_handle* h, int record, abd_frame_stats* stats) {
  if (!h) return ABD_ERR_INVALID;
  int ts = 0, st0 = 0, end = 0;
  char folder[4096];
  if (abd_get_trace(h, &ts, &st0, &end, folder, sizeof(folder)) != ABD_OK) return ABD_ERR_INVALID;
  if (end <= 0) return ABD_ERR_INVALID;  // no last frame: the loop would not end
  abd_frame_stats total;
  std::memset(&total, 0, sizeof(total));
  total.toi_min = 1.0;
  total.alpha_min = 1.0;
  int rc = ABD_OK;
  while (ts < end) {
    bool init = ts == 0;
    abd_frame_stats f;
    rc = abd_step(h, 0.0, 1, &f);
    ++ts;
    abd_set_trace(h, nullptr, ts, st0, end, nullptr, nullptr);
    total.frames += f.frames;
    total.newton_iters += f.newton_iters;
    total.ls_trials += f.ls_trials;
    total.pcg_iters += f.pcg_iters;
    total.n_pt = std::max(total.n_pt, f.n_pt);
    total.n_ee = std::max(total.n_ee, f.n_ee);
    total.n_vg = std::max(total.n_vg, f.n_vg);
    total.n_overlaps = std::max(total.n_overlaps, f.n_overlaps);
    total.kernel_launches += f.kernel_launches;
    total.toi_min = std::min(total.toi_min, f.toi_min);
    total.alpha_min = std::min(total.alpha_min, f.alpha_min);
    total.t_ipc_ms += f.t_ipc_ms;
    total.t_solver_ms += f.t_solver_ms;
    total.t_ccd_ms += f.t_ccd_ms;
    total.t_ls_ms += f.t_ls_ms;
    total.bytes_moved += f.bytes_moved;
    total.device_ms += f.device_ms;
    total.status = rc;
    if (rc != ABD_OK && rc != ABD_ERR_PCG_NOCONV && rc != ABD_ERR_LS_STALL) break;
    if (record) {
      int wr = abd_trace_save(h, folder, ts, init ? 1 : 0);
      if (wr != ABD_OK) {
        rc = wr;
        break;
      }
    }
  }
  if (stats) *stats = total;
  return rc;
}
