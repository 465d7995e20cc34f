"""Scene and config front end for the ABD contact path.

Reads and writes the reference's ``config.json`` keys (view/control.cpp:19-111) and its
scene schema (test_cases/spinning_cube.cpp:56-127: a JSON array of bodies with
``obj?``, ``omega``, ``p``, ``p_dot``, ``theta`` | ``euler``, ``mass?``), plus Wavefront
OBJ meshes. A scene is flattened into the structure-of-arrays layout the GPU engine
consumes: per-body state ``q0``/``dqdt`` (12 doubles: p, a1, a2, a3 where a_k are the
columns of A), ``mass``/``Ic`` and CSR-style offsets into rest vertices, edges and faces.

Seeded generators build the synthetic benchmark scenes (cubes, icosphere piles, torus
chains, batched scenes) with the reference's conventions: ground plane at y = -0.5
(geometry.cpp:57-62), ``Ic = mass / 12`` for meshes (affine_obj.h:10), ``mass < 0`` marks
a static body, and float-representable rest vertices (the reference stored them as
float through glm, view/mesh.h:17-19).
"""
from __future__ import annotations

import dataclasses
import json
import math
import os
from typing import Dict, List, Optional

import numpy as np

# ----------------------------------------------------------------------------------
# Config


@dataclasses.dataclass
class Config:
    """Step parameters, named after the reference's config.json keys."""

    dt: float = 1e-2
    kappa: float = 1e-4            # barrier stiffness ("kappa", control.cpp:107 -> barrier::kappa)
    dhat: float = 1e-4             # squared-distance activation (hard-coded in barrier.cpp:7)
    ortho_kappa: float = 1e9       # othogonal_energy.cpp:8
    ground_offset: float = 0.5     # vg_distance = y + 0.5 (geometry.cpp:60)
    mu: float = 0.0
    evh: float = 1e-3
    eps_x: float = 1e-3
    backoff: float = 0.8
    c1: float = 1e-4               # params_double.c1
    tol: float = 1e-2              # params_double.tol
    max_uk: float = 0.0            # params_double.max_uk
    dq_tol: float = 0.0            # params_double.dq_tol
    gravity: bool = True
    ls_grad_tol: float = 1e-3      # line_search.cpp:84 (hard-coded)
    max_iter: int = 1000
    max_iter_frame: int = 0        # Newton iterations per frame at most (0: unbounded, as the reference)
    autotune: bool = True          # narrow-phase launch variants chosen by timing (results unchanged)
    tri_direct: bool = True        # block-tridiagonal scenes solved by block Cholesky (solver "sparse")
    ground: bool = True
    pt: bool = True
    ee: bool = True
    psd: bool = True
    line_search: bool = True
    upper_bound: bool = True       # "uppper_bound" in the reference config
    vg_friction: bool = True
    pt_friction: bool = True
    ee_friction: bool = True
    clip: int = 0                  # params_int.clip
    iaabb: int = 3                 # odd: iAABB culling; even: spatial hash; > 1: iAABB step bound
    full_ccd: bool = True          # spatial-hash step bound: hashed trajectories (else the d_sqrt bound)
    safe_factor: float = 1.0       # spatial-hash distance scale
    sh_min_xyz: float = -10.0      # "spatial hashing": min_xyz, dx, xyz_bits, n_buffer
    sh_dx: float = 0.8
    sh_bits: int = 6
    sh_n_buffer: int = 512
    sh_fix_edge_trajectory: bool = False   # register edge trajectories by both ends (reference: start only)
    damping: bool = False          # "damping": {"enable", "alpha", "beta"} (mutils.cpp:106-115)
    damp_alpha: float = 5e-2
    damp_beta: float = 2.5e-2
    solver: str = "sparse"         # "solver": "sparse" (block-Jacobi PCG) or "dense" (per-scene dense Cholesky)
    # GPU solver controls (no reference counterpart: the reference factorizes directly)
    pcg_rel_tol: float = 1e-11
    pcg_max_iter: int = 5000
    pcg_refine: int = 0            # iterative-refinement passes after the PCG (true residual)
    pcg_refine_tol: float = 1e-8   # relative tolerance of each correction solve

    @property
    def gravity_y(self) -> float:
        return -9.8 if self.gravity else 0.0

    @property
    def d_sqrt(self) -> float:
        return math.sqrt(self.dhat)


def load_config(path: str) -> Config:
    """Parses a reference config.json (view/control.cpp:19-111)."""
    with open(path) as f:
        d = json.load(f)
    pd = d.get("params_double", {})
    pi = d.get("params_int", {})
    c = Config()
    c.dt = float(d.get("dt", c.dt))
    c.kappa = float(d.get("kappa", c.kappa))
    c.dhat = float(d.get("dhat", c.dhat))
    c.ortho_kappa = float(d.get("ortho_kappa", c.ortho_kappa))
    c.ground_offset = -float(d["ground_y"]) if "ground_y" in d else c.ground_offset
    c.mu = float(d.get("mu", c.mu))
    c.evh = float(d.get("evh", c.evh))
    c.eps_x = float(d.get("eps_x", c.eps_x))
    c.backoff = float(d.get("backoff", c.backoff))
    c.c1 = float(pd.get("c1", c.c1))
    c.tol = float(pd.get("tol", c.tol))
    c.max_uk = float(pd.get("max_uk", c.max_uk))
    c.dq_tol = float(pd.get("dq_tol", c.dq_tol))
    c.gravity = bool(d.get("gravity", c.gravity))
    c.max_iter = int(d.get("max_iter", c.max_iter))
    c.ground = bool(d.get("ground", c.ground))
    c.pt = bool(d.get("pt", c.pt))
    c.ee = bool(d.get("ee", c.ee))
    c.psd = bool(d.get("psd", c.psd))
    c.line_search = bool(d.get("line_search", c.line_search))
    c.upper_bound = bool(d.get("uppper_bound", d.get("upper_bound", c.upper_bound)))
    c.vg_friction = bool(d.get("vg_friction", c.vg_friction))
    c.pt_friction = bool(d.get("pt_friction", c.pt_friction))
    c.ee_friction = bool(d.get("ee_friction", c.ee_friction))
    c.clip = int(pi.get("clip", c.clip))
    c.iaabb = int(d.get("iaabb", c.iaabb))
    c.full_ccd = bool(d.get("full_ccd", c.full_ccd))
    c.safe_factor = float(d.get("safe_factor", c.safe_factor))
    sh = d.get("spatial hashing", {})
    c.sh_min_xyz = float(sh.get("min_xyz", c.sh_min_xyz))
    c.sh_dx = float(sh.get("dx", c.sh_dx))
    c.sh_bits = int(sh.get("xyz_bits", c.sh_bits))
    c.sh_n_buffer = int(sh.get("n_buffer", c.sh_n_buffer))
    c.sh_fix_edge_trajectory = bool(d.get("sh_fix_edge_trajectory", c.sh_fix_edge_trajectory))
    dmp = d.get("damping", {})
    c.damping = bool(dmp.get("enable", c.damping))
    c.damp_alpha = float(dmp.get("alpha", c.damp_alpha))
    c.damp_beta = float(dmp.get("beta", c.damp_beta))
    c.solver = str(d.get("solver", c.solver))
    c.pcg_rel_tol = float(d.get("pcg_rel_tol", c.pcg_rel_tol))
    c.pcg_max_iter = int(d.get("pcg_max_iter", c.pcg_max_iter))
    c.pcg_refine = int(d.get("pcg_refine", c.pcg_refine))
    c.max_iter_frame = int(d.get("max_iter_frame", c.max_iter_frame))
    c.autotune = bool(d.get("autotune", c.autotune))
    c.tri_direct = bool(d.get("tri_direct", c.tri_direct))
    c.pcg_refine_tol = float(d.get("pcg_refine_tol", c.pcg_refine_tol))
    return c


def config_to_json(c: Config) -> dict:
    """Reference-schema config dict (plus the keys this library adds)."""
    return {
        "dt": c.dt, "max_iter": c.max_iter, "gravity": c.gravity, "line_search": c.line_search,
        "col_set": True, "ee": c.ee, "pt": c.pt, "ground": c.ground, "uppper_bound": c.upper_bound,
        "mu": c.mu, "backoff": c.backoff, "eps_x": c.eps_x, "psd": c.psd, "iaabb": c.iaabb,
        "full_ccd": c.full_ccd, "safe_factor": c.safe_factor,
        "spatial hashing": {"min_xyz": c.sh_min_xyz, "max_xyz": -c.sh_min_xyz, "dx": c.sh_dx,
                            "n_buffer": c.sh_n_buffer, "xyz_bits": c.sh_bits, "set_size": 1},
        "sh_fix_edge_trajectory": c.sh_fix_edge_trajectory,
        "evh": c.evh, "vg_friction": c.vg_friction, "pt_friction": c.pt_friction,
        "ee_friction": c.ee_friction, "kappa": c.kappa, "solver": c.solver,
        "damping": {"enable": c.damping, "alpha": c.damp_alpha, "beta": c.damp_beta},
        "params_double": {"tol": c.tol, "c1": c.c1, "max_uk": c.max_uk, "dq_tol": c.dq_tol},
        "params_int": {"clip": c.clip, "thres": 100},
        "dhat": c.dhat, "ortho_kappa": c.ortho_kappa, "ground_y": -c.ground_offset,
        "pcg_rel_tol": c.pcg_rel_tol, "pcg_max_iter": c.pcg_max_iter,
        "pcg_refine": c.pcg_refine, "pcg_refine_tol": c.pcg_refine_tol, "max_iter_frame": c.max_iter_frame, "autotune": c.autotune,
        "tri_direct": c.tri_direct,
    }


# ----------------------------------------------------------------------------------
# Meshes


@dataclasses.dataclass
class Mesh:
    vertices: np.ndarray   # (n, 3) float64 (float32-representable)
    faces: np.ndarray      # (m, 3) int32
    edges: np.ndarray      # (k, 2) int32

    @property
    def volume(self) -> float:
        v = self.vertices[self.faces]
        return float(np.einsum("ij,ij->i", v[:, 0], np.cross(v[:, 1], v[:, 2])).sum() / 6.0)


def extract_edges(faces: np.ndarray) -> np.ndarray:
    """Unique (min, max) vertex pairs in lexicographic order (affine_obj.cpp:5-23)."""
    s = set()
    for a, b, c in faces.tolist():
        for u, v in ((a, b), (b, c), (a, c)):
            s.add((min(u, v), max(u, v)))
    return np.array(sorted(s), dtype=np.int32).reshape(-1, 2)


def cube_mesh() -> Mesh:
    """The reference's unit Cube (model/cube.h:4-70): vertex, triangle and edge order."""
    v = np.array([[-0.5, -0.5, -0.5], [-0.5, -0.5, 0.5], [-0.5, 0.5, -0.5], [-0.5, 0.5, 0.5],
                  [0.5, -0.5, -0.5], [0.5, -0.5, 0.5], [0.5, 0.5, -0.5], [0.5, 0.5, 0.5]])
    quads = [0, 1, 3, 2, 4, 5, 1, 0, 4, 0, 2, 6, 2, 3, 7, 6, 1, 5, 7, 3, 5, 4, 6, 7]
    tris = []
    for i in range(6):
        q = quads[4 * i: 4 * i + 4]
        tris += [q[0], q[1], q[2], q[2], q[3], q[0]]
    edges = []
    for i in range(3):
        di = 1 << (2 - i)
        for j in range(4):
            e0 = quads[i * 4 + j]
            edges += [e0, e0 + di]
    return Mesh(v.astype(np.float64), np.array(tris, np.int32).reshape(-1, 3),
                np.array(edges, np.int32).reshape(-1, 2))


def _f32(x: np.ndarray) -> np.ndarray:
    return x.astype(np.float32).astype(np.float64)


def icosphere_mesh(subdiv: int, radius: float = 0.5) -> Mesh:
    """Subdivided icosahedron projected to a sphere (10 * 4^s + 2 vertices)."""
    t = (1.0 + math.sqrt(5.0)) / 2.0
    verts = [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t], [0, -1, -t],
             [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]]
    faces = [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
             [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
             [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]]
    verts = [np.array(v, np.float64) / np.linalg.norm(v) for v in verts]
    for _ in range(subdiv):
        cache: Dict[tuple, int] = {}

        def mid(a: int, b: int) -> int:
            key = (min(a, b), max(a, b))
            if key not in cache:
                m = verts[a] + verts[b]
                verts.append(m / np.linalg.norm(m))
                cache[key] = len(verts) - 1
            return cache[key]

        nf = []
        for a, b, c in faces:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [[a, ab, ca], [b, bc, ab], [c, ca, bc], [ab, bc, ca]]
        faces = nf
    v = _f32(np.array(verts) * radius)
    f = np.array(faces, np.int32)
    return Mesh(v, f, extract_edges(f))


def torus_mesh(R: float = 1.0, r: float = 0.15, nu: int = 48, nv: int = 24) -> Mesh:
    """Torus in the xy-plane (axis z): nu segments around the ring, nv around the tube."""
    verts = []
    for i in range(nu):
        th = 2 * math.pi * i / nu
        for j in range(nv):
            ph = 2 * math.pi * j / nv
            rr = R + r * math.cos(ph)
            verts.append([rr * math.cos(th), rr * math.sin(th), r * math.sin(ph)])
    faces = []
    for i in range(nu):
        for j in range(nv):
            a = i * nv + j
            b = ((i + 1) % nu) * nv + j
            c = ((i + 1) % nu) * nv + (j + 1) % nv
            d = i * nv + (j + 1) % nv
            faces += [[a, b, c], [a, c, d]]
    f = np.array(faces, np.int32)
    return Mesh(_f32(np.array(verts)), f, extract_edges(f))


def read_obj(path: str) -> Mesh:
    vs, fs = [], []
    with open(path) as fh:
        for line in fh:
            t = line.split()
            if not t:
                continue
            if t[0] == "v":
                vs.append([float(x) for x in t[1:4]])
            elif t[0] == "f":
                idx = [int(x.split("/")[0]) - 1 for x in t[1:]]
                for k in range(1, len(idx) - 1):
                    fs.append([idx[0], idx[k], idx[k + 1]])
    f = np.array(fs, np.int32)
    return Mesh(np.array(vs, np.float64), f, extract_edges(f))


def write_obj(path: str, m: Mesh) -> None:
    with open(path, "w") as fh:
        for v in m.vertices:
            fh.write("v %r %r %r\n" % (float(v[0]), float(v[1]), float(v[2])))
        for a, b, c in m.faces:
            fh.write("f %d %d %d\n" % (a + 1, b + 1, c + 1))


# ----------------------------------------------------------------------------------
# Scenes


def rotation_zyx(a: float, b: float, c: float) -> np.ndarray:
    """geometry.cpp:248-264 `rotation(a, b, c)` = Rz(a) Ry(b) Rx(c)."""
    s1, s2, s3 = math.sin(a), math.sin(b), math.sin(c)
    c1, c2, c3 = math.cos(a), math.cos(b), math.cos(c)
    return np.array([[c1 * c2, c1 * s2 * s3 - c3 * s1, s1 * s3 + c1 * c3 * s2],
                     [c2 * s1, c1 * c3 + s1 * s2 * s3, c3 * s1 * s2 - c1 * s3],
                     [-s2, c2 * s3, c2 * c3]])


def skew_cols(w) -> np.ndarray:
    """geometry.h:28-35 `skew(w)`: the three 3-vectors stored as dA/dt columns."""
    a = w
    return np.array([-np.array([0, -a[2], a[1]]), -np.array([a[2], 0, -a[0]]),
                     -np.array([-a[1], a[0], 0])], np.float64)


@dataclasses.dataclass
class Scene:
    """Flattened scene: per-body state and CSR offsets into the mesh arrays."""

    q0: np.ndarray         # (nb, 12)
    dqdt: np.ndarray       # (nb, 12)
    mass: np.ndarray       # (nb,)
    Ic: np.ndarray         # (nb,)
    vert_off: np.ndarray   # (nb+1,) int32
    rest: np.ndarray       # (nv, 3)
    edge_off: np.ndarray   # (nb+1,)
    edges: np.ndarray      # (ne, 2) local vertex ids
    face_off: np.ndarray   # (nb+1,)
    faces: np.ndarray      # (nf, 3) local vertex ids
    scene_id: Optional[np.ndarray] = None   # (nb,) independent-scene index (batched runs)

    @property
    def n_bodies(self) -> int:
        return int(self.q0.shape[0])

    @property
    def n_vertices(self) -> int:
        return int(self.vert_off[-1])

    def copy(self) -> "Scene":
        return dataclasses.replace(self, **{f.name: (None if getattr(self, f.name) is None else
                                                     np.array(getattr(self, f.name)))
                                            for f in dataclasses.fields(self)})

    def body_range(self, b0: int, b1: int) -> "Scene":
        """Bodies [b0, b1) as a scene of their own (scene ids dropped)."""
        vo, eo, fo = self.vert_off, self.edge_off, self.face_off
        return Scene(q0=np.array(self.q0[b0:b1]), dqdt=np.array(self.dqdt[b0:b1]), mass=np.array(self.mass[b0:b1]),
                     Ic=np.array(self.Ic[b0:b1]), vert_off=(vo[b0:b1 + 1] - vo[b0]).astype(np.int32),
                     rest=np.array(self.rest[vo[b0]:vo[b1]]), edge_off=(eo[b0:b1 + 1] - eo[b0]).astype(np.int32),
                     edges=np.array(self.edges[eo[b0]:eo[b1]]), face_off=(fo[b0:b1 + 1] - fo[b0]).astype(np.int32),
                     faces=np.array(self.faces[fo[b0]:fo[b1]]), scene_id=None)

    def scenes_of_rank(self, rank: int, world: int) -> "Scene":
        """The scenes of one rank when a batch is sharded by scene over `world` processes:
        scene k goes to rank k % world (independent scenes need no exchange), in order, with
        scene ids renumbered from 0."""
        ranges = [r for k, r in enumerate(self.scene_ranges()) if k % world == rank]
        parts = [self.body_range(b0, b1) for b0, b1 in ranges]
        if not parts:
            raise ValueError("rank %d of %d holds no scene" % (rank, world))
        out = parts[0]
        for k, p in enumerate(parts[1:], 1):
            out = concat_scenes(out, p)
        if len(parts) > 1 or self.scene_id is not None:
            sid = np.concatenate([np.full(p.n_bodies, k, np.int32) for k, p in enumerate(parts)])
            out = dataclasses.replace(out, scene_id=sid)
        return out

    def scene_ranges(self):
        """(first body, end body) of each scene, in order (one range without scene ids)."""
        if self.scene_id is None:
            return [(0, self.n_bodies)]
        sid = np.asarray(self.scene_id)
        cuts = [0] + [int(i) for i in np.nonzero(sid[1:] != sid[:-1])[0] + 1] + [self.n_bodies]
        return list(zip(cuts[:-1], cuts[1:]))


def concat_scenes(a: "Scene", b: "Scene") -> "Scene":
    """Bodies of a then b as one scene (scene ids dropped)."""
    return Scene(q0=np.concatenate([a.q0, b.q0]), dqdt=np.concatenate([a.dqdt, b.dqdt]),
                 mass=np.concatenate([a.mass, b.mass]), Ic=np.concatenate([a.Ic, b.Ic]),
                 vert_off=np.concatenate([a.vert_off, a.vert_off[-1] + b.vert_off[1:]]).astype(np.int32),
                 rest=np.concatenate([a.rest, b.rest]),
                 edge_off=np.concatenate([a.edge_off, a.edge_off[-1] + b.edge_off[1:]]).astype(np.int32),
                 edges=np.concatenate([a.edges, b.edges]),
                 face_off=np.concatenate([a.face_off, a.face_off[-1] + b.face_off[1:]]).astype(np.int32),
                 faces=np.concatenate([a.faces, b.faces]), scene_id=None)


class SceneBuilder:
    def __init__(self):
        self.meshes: List[Mesh] = []
        self.bodies: List[dict] = []

    def add(self, mesh: Mesh, p, R=None, p_dot=(0, 0, 0), omega=(0, 0, 0), mass=None, Ic=None, scene_id=0):
        R = np.eye(3) if R is None else np.asarray(R, np.float64)
        q = np.zeros(12)
        q[0:3] = p
        for k in range(3):
            q[3 + 3 * k: 6 + 3 * k] = R[:, k]
        qd = np.zeros(12)
        qd[0:3] = p_dot
        qd[3:12] = skew_cols(np.asarray(omega, np.float64)).reshape(-1)
        m = 1000.0 if mass is None else float(mass)
        ic = (m / 12.0) if Ic is None else float(Ic)
        self.meshes.append(mesh)
        self.bodies.append(dict(q=q, qd=qd, m=m, ic=ic, sid=scene_id))
        return self

    def build(self) -> Scene:
        nb = len(self.bodies)
        vo, eo, fo = [0], [0], [0]
        for m in self.meshes:
            vo.append(vo[-1] + len(m.vertices))
            eo.append(eo[-1] + len(m.edges))
            fo.append(fo[-1] + len(m.faces))
        return Scene(
            q0=np.array([b["q"] for b in self.bodies]).reshape(nb, 12),
            dqdt=np.array([b["qd"] for b in self.bodies]).reshape(nb, 12),
            mass=np.array([b["m"] for b in self.bodies]),
            Ic=np.array([b["ic"] for b in self.bodies]),
            vert_off=np.array(vo, np.int32),
            rest=np.concatenate([m.vertices for m in self.meshes]).reshape(-1, 3),
            edge_off=np.array(eo, np.int32),
            edges=np.concatenate([m.edges for m in self.meshes]).reshape(-1, 2).astype(np.int32),
            face_off=np.array(fo, np.int32),
            faces=np.concatenate([m.faces for m in self.meshes]).reshape(-1, 3).astype(np.int32),
            scene_id=np.array([b["sid"] for b in self.bodies], np.int32),
        )


def load_scene(path: str, mesh_dir: Optional[str] = None) -> Scene:
    """Reads a reference-schema scene JSON (spinning_cube.cpp:56-127)."""
    with open(path) as f:
        data = json.load(f)
    base = mesh_dir or os.path.dirname(os.path.abspath(path))
    cache: Dict[str, Mesh] = {}
    sb = SceneBuilder()
    for it in data:
        if "obj" in it:
            fn = it["obj"]
            if fn not in cache:
                cache[fn] = read_obj(fn if os.path.isabs(fn) else os.path.join(base, fn))
            mesh = cache[fn]
        else:
            mesh = cube_mesh()
        omega = it.get("omega", [0.0, 0.0, 20.0])
        if "euler" in it:
            ds = it["euler"]
            R = rotation_zyx(ds[2] / 180.0 * math.pi, ds[1] / 180.0 * math.pi, ds[0] / 180.0 * math.pi)
        else:
            th = it.get("theta", 0.0) / 180.0 * math.pi
            s, c = math.sin(th), math.cos(th)
            R = np.eye(3)
            R[0, 0] = c; R[1, 1] = c; R[0, 1] = -s; R[1, 0] = s
        m = it.get("mass", None)
        sb.add(mesh, it["p"], R, it.get("p_dot", [0, 0, 0]), omega,
               mass=None if m is None else float(m))
    return sb.build()


def scene_to_json(entries: List[dict], path: str) -> None:
    with open(path, "w") as f:
        json.dump(entries, f, indent=1)


# ----------------------------------------------------------------------------------
# Synthetic benchmark scenes (seeded). y positions are given relative to a ground at
# y = 0 and shifted by -0.5 onto the reference's ground plane.

GROUND_SHIFT = -0.5


def random_rotation(rng: np.random.Generator) -> np.ndarray:
    """Uniform random rotation (Shoemake quaternion)."""
    u1, u2, u3 = rng.random(3)
    q = np.array([math.sqrt(1 - u1) * math.sin(2 * math.pi * u2), math.sqrt(1 - u1) * math.cos(2 * math.pi * u2),
                  math.sqrt(u1) * math.sin(2 * math.pi * u3), math.sqrt(u1) * math.cos(2 * math.pi * u3)])
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def cube_stack(n: int = 10, gap: float = 0.1, seed: int = 0) -> Scene:
    """n unit cubes stacked along y with `gap` between them and above the ground, each
    with a random yaw (rotation about y)."""
    rng = np.random.default_rng(seed)
    sb = SceneBuilder()
    cube = cube_mesh()
    for k in range(n):
        yaw = rng.random() * 2 * math.pi
        R = rotation_zyx(0.0, yaw, 0.0)
        y = gap + 0.5 + k * (1.0 + gap) + GROUND_SHIFT
        sb.add(cube, (0.0, y, 0.0), R)
    return sb.build()


def sphere_pile(nx: int = 16, nz: int = 16, ny: int = 4, spacing: float = 1.1, subdiv: int = 3,
                radius: float = 0.5, jitter: float = 0.02, vel_sigma: float = 0.5, seed: int = 0,
                density: float = 1000.0) -> Scene:
    """Icospheres on an nx x ny x nz grid (spacing apart, lowest layer spacing/2 above
    the ground), uniform random rotation, uniform +-jitter position noise and initial
    velocity N(0, vel_sigma^2) per axis."""
    rng = np.random.default_rng(seed)
    mesh = icosphere_mesh(subdiv, radius)
    m = density * mesh.volume
    sb = SceneBuilder()
    for iy in range(ny):
        for ix in range(nx):
            for iz in range(nz):
                R = random_rotation(rng)
                j = rng.uniform(-jitter, jitter, 3)
                v = rng.normal(0.0, vel_sigma, 3)
                p = np.array([(ix - (nx - 1) / 2) * spacing, spacing / 2 + iy * spacing + GROUND_SHIFT,
                              (iz - (nz - 1) / 2) * spacing]) + j
                sb.add(mesh, p, R, p_dot=v, mass=m)
    return sb.build()


def torus_chain(n: int = 200, R: float = 1.0, r: float = 0.15, gap: float = 0.1, omega_sigma: float = 1.0,
                seed: int = 0, density: float = 1000.0, nu: int = 48, nv: int = 24) -> Scene:
    """Interlocked torus links along x; odd links rotated 90 degrees about x; link 0 is
    static; every other link gets angular velocity N(0, omega_sigma^2) per axis."""
    rng = np.random.default_rng(seed)
    mesh = torus_mesh(R, r, nu, nv)
    m = density * mesh.volume
    L = 2 * R - 2 * r - gap
    sb = SceneBuilder()
    Rx = rotation_zyx(0.0, 0.0, math.pi / 2)
    for k in range(n):
        Rk = Rx if (k % 2) else np.eye(3)
        om = rng.normal(0.0, omega_sigma, 3) if (k % 2 == 1) else np.zeros(3)
        sb.add(mesh, (k * L, 10.0, 0.0), Rk, omega=om, mass=(-1.0 if k == 0 else m))
    return sb.build()


def batched_scenes(n_scenes: int = 256, seed: int = 0, lo: int = 4, hi: int = 128, spacing: float = 4.0,
                   vel_sigma: float = 0.5) -> Scene:
    """Independent scenes side by side (scene_id per body): body counts
    clip(round(lognormal(3, 1)), lo, hi), 50/50 unit cubes and subdivision-2
    icospheres, each scene a non-overlapping column above the ground."""
    rng = np.random.default_rng(seed)
    cube, ico = cube_mesh(), icosphere_mesh(2, 0.5)
    m_ico = 1000.0 * ico.volume
    sb = SceneBuilder()
    side = int(math.ceil(math.sqrt(n_scenes)))
    for s in range(n_scenes):
        nb = int(np.clip(round(rng.lognormal(3.0, 1.0)), lo, hi))
        cx, cz = (s % side) * spacing, (s // side) * spacing
        for k in range(nb):
            is_cube = rng.random() < 0.5
            R = random_rotation(rng)
            v = rng.normal(0.0, vel_sigma, 3)
            y = 0.1 + 0.5 * math.sqrt(3) + k * (math.sqrt(3) + 0.1) + GROUND_SHIFT
            if is_cube:
                sb.add(cube, (cx, y, cz), R, p_dot=v, scene_id=s)
            else:
                sb.add(ico, (cx, y, cz), R, p_dot=v, mass=m_ico, scene_id=s)
    return sb.build()


def diff_grid(seed: int = 0, n: int = 4, spacing: float = 1.2, lift: float = 0.6) -> Scene:
    """n^3 subdivision-2 icospheres on an n x n x n grid (64 with spacing 1.2 by default),
    the lowest layer `lift` above the ground."""
    rng = np.random.default_rng(seed)
    ico = icosphere_mesh(2, 0.5)
    m = 1000.0 * ico.volume
    sb = SceneBuilder()
    c = (n - 1) / 2
    for iy in range(n):
        for ix in range(n):
            for iz in range(n):
                p = ((ix - c) * spacing, lift + iy * spacing + GROUND_SHIFT, (iz - c) * spacing)
                sb.add(ico, p, random_rotation(rng), mass=m)
    return sb.build()


def diff_targets(n_bodies: int = 64, seed: int = 0) -> np.ndarray:
    """Seeded targets of the differentiable-rollout loss: uniform in
    [-2, 2] x [0.5, 1.5] x [-2, 2] above the ground (shifted to the reference's ground)."""
    rng = np.random.default_rng(seed)
    t = rng.uniform((-2.0, 0.5, -2.0), (2.0, 1.5, 2.0), (n_bodies, 3))
    t[:, 1] += GROUND_SHIFT
    return t


def workload_config(name: str) -> Config:
    """Physical parameters of the named synthetic workloads."""
    c = Config()
    if name in ("cubes", "pile", "batched", "diff"):
        c.dt, c.dhat, c.kappa, c.mu, c.tol = 1e-2, 1e-3, 1e-4, 0.1, 1e-4
        if name == "diff":
            # mu 0.3: the lagged friction's Newton iteration cycles on some impact frames
            # (it never reaches tol), so those frames stop after 100 iterations
            c.mu = 0.3
            c.max_iter_frame = 100
        elif name == "pile":
            # from rest with seed 0, frames 32 and 77 of the 200 cycle: they stop after 100
            c.max_iter_frame = 100
        elif name == "batched":
            # among 256 scenes a frame whose lagged friction cycles turns up now and then
            # (scene 95 of the seeded batch takes 260 iterations on frame 34); a batch
            # steps until its slowest scene stops, so such frames stop after 100
            c.max_iter_frame = 100
    elif name == "chain":
        c.dt, c.dhat, c.kappa, c.mu, c.tol, c.ground = 5e-3, 1e-4, 1e-4, 0.2, 1e-4, False
        # the lagged friction's Newton iteration cycles on a few frames of the 300 (170
        # and 267 from rest with seed 0): those frames stop after 100 iterations
        c.max_iter_frame = 100
    c.max_iter = 1 << 30
    return c
