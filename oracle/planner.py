"""ORACLE - test infrastructure, not product code.

The oracle's own restatement of the reference's plan construction, so that a
CPU run of the reference path (bench.py's reference arm and cpu_baseline leg)
uses no engine code at all. Imported only by tests/, __graft_entry__.smoke()
and those two bench legs, always as the checker or the CPU baseline.

  read_mesh      the .mesh text format (surface::loadLattice, src/interpLib.C:1144-1300)
  orient         triangle discovery in the reference's order (constructTriangles,
                 src/interpLib.C:7222-7290) and triangle senses propagated from
                 triangle 0 across shared edges (src/interpLib.C:1780-1830); the
                 oriented vertex rings follow from the senses
  faces          per-face control-point lists (point_list, src/interpLib.C:5490-5553)
                 and their lattice images (r_pbc, src/interpLib.C:6028-6045)
  set_reference  setg0: g0 and RuRv0 at every quadrature point, the face areas
                 and the whole-lipid leaflet fill (src/interpLib.C:2969-3195)
  icosphere      the synthetic vesicle of the benchmark workload: icosahedron,
                 Loop-subdivided, radial Philox noise (the same file the
                 workload's generator writes)

The basis rows and quadrature weights are the reference's own: its plan dump
committed in tests/golden/ico2_plain.npz holds the regular rows (15 points)
and the valence-5 rows (16 points), which every face of an icosahedral mesh
uses. Meshes with valence-7 vertices are therefore not planned here.
"""
from __future__ import annotations

import ctypes as C
import math
from pathlib import Path

import numpy as np

from oracle import bridge as OB

ROOT = Path(__file__).resolve().parent.parent
BASIS_DUMP = ROOT / "tests" / "golden" / "ico2_plain.npz"

HALF_LIPID = 0.5 * 65.0     # area_per_lipid_av / 2 (src/interpLib.C:3157-3172)
# built-in lipid library (src/lipid_composition.C:18-32): name -> (c0 1/A, APL A^2)
LIBRARY = {"ZERO": (0.0, 68.3), "POPC": (-1.0 / 87.3, 68.3), "DOPE": (-1.0 / 29.4, 63.4),
           "POPE": (-1.0 / 29.4, 58.8), "DOPC": (-1.0 / 87.3, 69.7), "CHOL": (-1.0 / 27.2, 31.0),
           "CHL1": (-1.0 / 27.2, 31.0), "DOG": (-1.0 / 11.5, 59.0), "DOPS": (1.0 / 144.0, 71.6),
           "CER180": (0.0, 59.0), "SSM": (0.0, 59.0), "PSM": (0.0, 59.0)}


# ------------------------------------------------------------------ mesh text

class MeshText:
    """What a .mesh file holds: positions, box vectors, file-order rings."""

    def __init__(self, r, box, rings, fix_sense=1):
        self.r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
        self.box = np.asarray(box, dtype=np.float64).reshape(3, 3)
        self.rings = [list(x) for x in rings]
        self.fix_sense = fix_sense
        self.nv = len(self.rings)


def read_mesh(path) -> MeshText:
    """The reference's .mesh format: a '3D' (or '2D', Lz = 1e6) header, the box
    vectors, an optional 'sense N' line, then 'id x y z valence n1 .. nval'."""
    lines = Path(path).read_text().splitlines()
    vec3 = lines[0].strip().upper().startswith("3D")
    nvec = 3 if vec3 else 2
    box = [[float(t) for t in lines[1 + d].split()[:3]] for d in range(nvec)]
    if not vec3:
        box.append([0.0, 0.0, 1e6])
    ln, fix_sense = 1 + nvec, 1
    if ln < len(lines) and lines[ln].strip().lower().startswith("sense"):
        fix_sense = int(lines[ln].split()[1])
        ln += 1
    r, rings = [], []
    for line in lines[ln:]:
        f = line.split()
        if not f:
            continue
        if f[0].lower().startswith("ntri"):
            break
        if not f[0].lstrip("-").isdigit():
            raise ValueError("protein points are not planned here")
        val = int(f[4])
        if not 5 <= val <= 7:
            raise ValueError("vertex valence must be between 5 and 7")
        r.append([float(f[1]), float(f[2]), float(f[3])])
        rings.append([int(t) for t in f[5:5 + val]])
    return MeshText(r, box, rings, fix_sense)


# ------------------------------------------------------------------ orientation

def _compare_sense(c1: int, c2: int) -> int:
    """Relative sense of two triangles sharing an edge; edge codes (a,b)=2,
    (a,c)=1, (b,c)=0 of each triangle's sorted ids (src/interpLib.C:110-121)."""
    return 1 if (c1 == 1) != (c2 == 1) else -1


def orient(m: MeshText) -> list[list[int]]:
    """Oriented rings: each vertex's ring starts at its first file-order
    neighbour and turns the way the senses fixed from triangle 0 say."""
    rings = m.rings
    ringset = [set(x) for x in rings]
    tris = []
    for i in range(m.nv):
        for j in rings[i]:
            if j < i:
                continue
            for k in rings[j]:
                if k == i or k < j:
                    continue
                if i in ringset[k]:
                    tris.append((i, j, k))
    edges: dict[tuple[int, int], list] = {}
    for t, (a, b, c) in enumerate(tris):
        for key, code in (((a, b), 2), ((a, c), 1), ((b, c), 0)):
            edges.setdefault(key, []).append((t, code))
    sense = [0] * len(tris)
    sense[0] = m.fix_sense
    adj = [[] for _ in tris]
    for fc in edges.values():
        if len(fc) >= 2:
            (f1, c1), (f2, c2) = fc[0], fc[1]
            s = _compare_sense(c1, c2)
            adj[f1].append((f2, s))
            adj[f2].append((f1, s))
    queue = [0]
    for t in queue:
        for u, s in adj[t]:
            want = sense[t] * s
            if sense[u] == 0:
                sense[u] = want
                queue.append(u)
            elif sense[u] != want:
                raise ValueError("surface is not orientable")
    succ = [dict() for _ in range(m.nv)]
    for (a, b, c), s in zip(tris, sense):
        if s == 0:
            raise ValueError("a triangle is not reachable from triangle 0")
        if s < 0:
            b, c = c, b
        succ[a][c] = b
        succ[b][a] = c
        succ[c][b] = a
    out = []
    for i in range(m.nv):
        ring = [rings[i][0]]
        for _ in range(len(rings[i]) - 1):
            ring.append(succ[i][ring[-1]])
        if succ[i][ring[-1]] != ring[0]:
            raise ValueError(f"vertex {i}: ring does not close")
        out.append(ring)
    return out


# ------------------------------------------------------------------ faces

def _min_image(dr: np.ndarray, box: np.ndarray) -> np.ndarray:
    """Lattice shift (-1, 0 or +1 per box vector) taking dr to its nearest image."""
    shift = np.zeros(3, dtype=np.int64)
    t = dr.copy()
    improved = True
    while improved:
        improved = False
        best = t @ t
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    cand = t + dx * box[0] + dy * box[1] + dz * box[2]
                    if cand @ cand < best - 1e-7:
                        best, tbest, sbest = cand @ cand, cand, (dx, dy, dz)
                        improved = True
        if improved:
            t = tbest
            shift += sbest
    return shift


def faces(m: MeshText, rings: list[list[int]]):
    """Regular faces (cp [n,12], img [n,12,3]) and irregular faces (valence,
    cp [n,13], img [n,13,3]) in the reference's face order."""
    reg_cp, reg_img, irr_val, irr_cp, irr_img = [], [], [], [], []
    pos = {}
    for i, ring in enumerate(rings):
        pos.update({(i, v): e for e, v in enumerate(ring)})
    free = 0.25 * min(float(np.sum((dx * m.box[0] + dy * m.box[1] + dz * m.box[2]) ** 2))
                      for dx in (-1, 0, 1) for dy in (-1, 0, 1) for dz in (-1, 0, 1) if dx or dy or dz)
    for i, ring in enumerate(rings):
        val = len(ring)
        for e in range(val):
            j, k = ring[e], ring[(e + 1) % val]
            if j < i or k < i:
                continue
            rj, rk = rings[j], rings[k]
            if len(rj) != 6 or len(rk) != 6:
                raise ValueError("a face touches two irregular vertices")
            ej, ek = pos[(j, i)], pos[(k, i)]
            cp = [i, k, j] + [ring[(e - q) % val] for q in range(1, val - 1)]
            cp += [rk[(ek - 2) % 6], rk[(ek + 3) % 6], rk[(ek + 2) % 6], rj[(ej + 3) % 6], rj[(ej + 2) % 6]]
            img = []
            for v in cp:
                dr = m.r[v] - m.r[i]
                img.append(np.zeros(3, dtype=np.int64) if dr @ dr < free else _min_image(dr, m.box))
            if val == 6:
                reg_cp.append(cp)
                reg_img.append(img)
            else:
                irr_val.append(val)
                irr_cp.append(cp + [0] * (13 - len(cp)))
                irr_img.append(img + [np.zeros(3, dtype=np.int64)] * (13 - len(img)))
    return (np.array(reg_cp, dtype=np.int32).reshape(-1, 12), np.array(reg_img, dtype=np.int8).reshape(-1, 12, 3),
            np.array(irr_val, dtype=np.int32), np.array(irr_cp, dtype=np.int32).reshape(-1, 13),
            np.array(irr_img, dtype=np.int8).reshape(-1, 13, 3))


# ------------------------------------------------------------------ reference state

def parse_lipids(text: str | None):
    """'lipid library NAME APL c0' and 'lipid outer|inner NAME parts' lines
    (src/lipid_composition.C:47-300) -> [(name, c0, apl, outer, inner)]."""
    lib = dict(LIBRARY)
    rows = [ln.split() for ln in (text or "").splitlines()]
    for f in rows:
        if len(f) >= 5 and f[0].lower() == "lipid" and f[1].lower() == "library":
            lib[f[2].upper()] = (float(f[4]), float(f[3]))
    types: dict[str, list] = {}
    for f in rows:
        if len(f) >= 4 and f[0].lower() == "lipid" and f[1].lower() in ("outer", "inner"):
            c0, apl = lib[f[2].upper()]
            t = types.setdefault(f[2].upper(), [f[2].upper(), c0, apl, 0.0, 0.0])
            t[3 if f[1].lower() == "outer" else 4] += float(f[3])
    out = list(types.values()) or [["ZERO", 0.0, 68.3, 0.0, 0.0]]
    if sum(t[3] for t in out) == 0:
        out[0][3] = 1.0
    if sum(t[4] for t in out) == 0:
        out[0][4] = 1.0
    return [tuple(t) for t in out]


def _fill(area: float, apl: float) -> float:
    """Leaflet area of whole lipids added until it exceeds area - 32.5
    (src/interpLib.C:3157-3195; one lipid type per leaflet, so no draws)."""
    n = 1
    while not n * apl > area - HALF_LIPID:
        n += 1
    return n * apl


def reference_basis():
    """The reference's basis rows [kind w,u,v,uu,uv,vv][pt][cp] and weights:
    (regular rows, weights), (valence-5 rows, weights)."""
    d = np.load(BASIS_DUMP)
    return ((np.ascontiguousarray(d["reg_rows"].transpose(1, 0, 2)), np.array(d["reg_w"])),
            (np.ascontiguousarray(d["irr_rows"].transpose(1, 0, 2)), np.array(d["irr_w"])))


def _points(rows, w, X, dudv):
    """g0, RuRv0 at every point and the face areas (setg0, src/interpLib.C:3060-3113)."""
    Ru = np.einsum("pj,fjc->fpc", rows[1], X)
    Rv = np.einsum("pj,fjc->fpc", rows[2], X)
    uu, uv, vv = (Ru * Ru).sum(-1), (Ru * Rv).sum(-1), (Rv * Rv).sum(-1)
    g = np.sqrt(uu * vv - uv * uv)
    return g, uv / np.sqrt(uu * vv), (g * dudv * w[None, :]).sum(1)


class Surface:
    """The oracle's plan of one mesh and the oracle_surface the C restatement
    evaluates (energy, gradient) over it."""

    def __init__(self, m: MeshText, kc: float, KA: float = 0.215, kg: float = 0.0, k_reg: float = 0.0,
                 lipids: str | None = None, topology: dict | None = None):
        """topology: a cache of the face lists, shared by meshes with one
        connectivity whose control points all stay in their home images (the
        vesicles of one subdivision level); filled on first use."""
        self.nv = m.nv
        if topology:
            self.reg_cp, self.reg_img, self.irr_val, self.irr_cp, self.irr_img = topology["faces"]
        else:
            self.reg_cp, self.reg_img, self.irr_val, self.irr_cp, self.irr_img = faces(m, orient(m))
            if topology is not None:
                topology["faces"] = (self.reg_cp, self.reg_img, self.irr_val, self.irr_cp, self.irr_img)
        if np.any(self.irr_val != 5):
            raise ValueError("only regular and valence-5 faces are planned here")
        (R6, w6), (R5, w5) = reference_basis()
        types = parse_lipids(lipids)
        if len(types) > 1 and (sum(t[3] > 0 for t in types) > 1 or sum(t[4] > 0 for t in types) > 1):
            raise ValueError("one lipid type per leaflet only")
        box = m.box

        def local(cp, img):
            return m.r[cp] + np.einsum("fjd,dc->fjc", img.astype(np.float64), box)

        self.reg_g0, self.reg_rr0, reg_area = _points(R6, w6, local(self.reg_cp, self.reg_img), 0.5)
        nirr = len(self.irr_val)
        if nirr:
            self.irr_g0, self.irr_rr0, irr_area = _points(R5, w5, local(self.irr_cp[:, :11], self.irr_img[:, :11]),
                                                          1.0)
        else:
            self.irr_g0 = self.irr_rr0 = np.zeros((0, 16))
            irr_area = np.zeros(0)
        nt = len(types)
        self.lipid_c0 = np.array([t[1] for t in types])

        def leaflets(area):
            o, i = np.zeros((len(area), nt)), np.zeros((len(area), nt))
            for x, t in enumerate(types):
                if t[3] > 0:
                    o[:, x] = [_fill(a, t[2]) for a in area]
                if t[4] > 0:
                    i[:, x] = [_fill(a, t[2]) for a in area]
            return o, i

        self.reg_outer, self.reg_inner = leaflets(reg_area)
        self.irr_outer, self.irr_inner = leaflets(irr_area)
        s = OB.OracleSurface()
        keep = []

        def k(a, ct=C.c_double):
            a = np.ascontiguousarray(a)
            keep.append(a)
            return a.ctypes.data_as(C.POINTER(ct))

        s.nv = m.nv
        s.box[:] = box.reshape(-1).tolist()
        s.kc, s.KA, s.kg, s.k_reg = kc, KA, kg, k_reg
        s.ntypes = nt
        s.lipid_c0 = k(self.lipid_c0)
        s.nreg = len(self.reg_cp)
        s.reg_cp, s.reg_img = k(self.reg_cp, C.c_int), k(self.reg_img, C.c_int8)
        s.reg_rows, s.reg_w = k(R6), k(w6)
        s.reg_g0, s.reg_rr0 = k(self.reg_g0), k(self.reg_rr0)
        s.reg_outer, s.reg_inner = k(self.reg_outer), k(self.reg_inner)
        s.nirr = nirr
        s.irr_val, s.irr_cp, s.irr_img = k(self.irr_val, C.c_int), k(self.irr_cp, C.c_int), k(self.irr_img, C.c_int8)
        s.irr_rows5, s.irr_w5 = k(R5), k(w5)
        s.irr_rows7, s.irr_w7 = None, None
        s.irr_g0, s.irr_rr0 = k(self.irr_g0), k(self.irr_rr0)
        s.irr_outer, s.irr_inner = k(self.irr_outer), k(self.irr_inner)
        self.s, self._keep = s, keep
        self.positions = np.concatenate([m.r.reshape(-1), np.ones(3)])

    def energy(self, r) -> float:
        r = np.ascontiguousarray(r, dtype=np.float64)
        return OB.lib().oracle_energy(C.byref(self.s), r.ctypes.data_as(C.POINTER(C.c_double)), None, None)

    def grad(self, r) -> np.ndarray:
        r = np.ascontiguousarray(r, dtype=np.float64)
        g = np.zeros(3 * self.nv + 3)
        OB.lib().oracle_grad(C.byref(self.s), r.ctypes.data_as(C.POINTER(C.c_double)),
                             g.ctypes.data_as(C.POINTER(C.c_double)))
        return g


# ------------------------------------------------------------------ the workload's vesicles

def _philox(c0, c1, c2, c3, k0, k1):
    """Philox4x32-10 (Salmon et al., SC'11) on uint64 arrays holding 32-bit words."""
    M = 0xFFFFFFFF
    c = [np.asarray(x, dtype=np.uint64) & M for x in (c0, c1, c2, c3)]
    k0, k1 = np.uint64(k0 & M), np.uint64(k1 & M)
    for _ in range(10):
        p0 = np.uint64(0xD2511F53) * c[0]
        p1 = np.uint64(0xCD9E8D57) * c[2]
        c = [((p1 >> np.uint64(32)) ^ c[1] ^ k0) & M, p1 & M, ((p0 >> np.uint64(32)) ^ c[3] ^ k1) & M, p0 & M]
        k0 = (k0 + np.uint64(0x9E3779B9)) & M
        k1 = (k1 + np.uint64(0xBB67AE85)) & M
    return c


def _u53(a, b):
    m = ((a >> np.uint64(5)) << np.uint64(26)) | (b >> np.uint64(6))
    return (m.astype(np.float64) + 0.5) / 9007199254740992.0


def icosphere(level: int, R: float, sigma: float, seed: int) -> MeshText:
    """Icosahedron (12 unit vertices (0, +-1, +-phi) cyclically, faces oriented
    outward), Loop-subdivided `level` times (one new vertex per edge at the
    normalised midpoint, appended in face order), radius R * (1 + N(0,
    sigma/R)) per vertex from Philox keyed by (seed, vertex); box 3R; rings
    counter-clockwise from the smallest-id neighbour."""
    phi = (1.0 + math.sqrt(5.0)) / 2.0
    p = np.array([[0, 1, phi], [0, -1, phi], [0, 1, -phi], [0, -1, -phi], [1, phi, 0], [-1, phi, 0],
                  [1, -phi, 0], [-1, -phi, 0], [phi, 0, 1], [-phi, 0, 1], [phi, 0, -1], [-phi, 0, -1]], float)
    p /= np.linalg.norm(p, axis=1, keepdims=True)
    pts = [tuple(x) for x in p]
    d2 = lambda a, b: float(np.sum((p[a] - p[b]) ** 2))  # noqa: E731
    emin = min(d2(a, b) for a in range(12) for b in range(a + 1, 12))
    tris = []
    for a in range(12):
        for b in range(a + 1, 12):
            for c in range(b + 1, 12):
                if max(d2(a, b), d2(a, c), d2(b, c)) > emin * 1.01:
                    continue
                if np.dot(np.cross(p[b] - p[a], p[c] - p[a]), p[a]) > 0:
                    tris.append((a, b, c))
                else:
                    tris.append((a, c, b))
    for _ in range(level):
        mid: dict[tuple[int, int], int] = {}

        def midpoint(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                q = 0.5 * (np.array(pts[a]) + np.array(pts[b]))
                pts.append(tuple(q / np.linalg.norm(q)))
                mid[key] = len(pts) - 1
            return mid[key]

        nt = []
        for a, b, c in tris:
            ab, bc, ca = midpoint(a, b), midpoint(b, c), midpoint(c, a)
            nt += [(a, ab, ca), (ab, b, bc), (ca, bc, c), (ab, bc, ca)]
        tris = nt
    P = np.array(pts)
    nv = len(P)
    o = _philox(np.arange(nv), 0, 0, 0x6D657368, seed, seed >> 32)
    u1, u2 = _u53(o[0], o[1]), _u53(o[2], o[3])
    rad = R + sigma * np.sqrt(-2.0 * np.log(u1)) * np.cos(2.0 * math.pi * u2)
    nxt = [dict() for _ in range(nv)]
    for a, b, c in tris:
        nxt[a][b] = c
        nxt[b][c] = a
        nxt[c][a] = b
    rings = []
    for v in range(nv):
        start = min(nxt[v])
        ring, cur = [start], nxt[v][start]
        while cur != start:
            ring.append(cur)
            cur = nxt[v][cur]
        rings.append(ring)
    return MeshText(rad[:, None] * P, np.eye(3) * 3.0 * R, rings)
