"""Synthetic meshes and the setup data the Galerkin hot path reads.

Host-side setup, run once per mesh (the reference does this in src/geometry, src/dofmap, src/wake and
src/meshtools). Only what the hot path consumes is produced:

- ``Geometry``: node coordinates ``x`` (nnode x 3), triangles ``tris`` (ntri x 3, 0-based, counterclockwise about the
  outward normal) and ``touch_pairs`` (SurfaceGeometry fields read by assemble.jl:383-386);
- ``DOFMapping``: slots, ``corner_slot``, the constraint matrix ``C`` (nslot x nq), the Kutta rows ``K``
  (nte x nq), the wake trailing edge, ``slot_area``, ``slot_body``, ``body_q``, ``body_closed``
  (src/dofmap/types.jl:73-93);
- ``RigidWake``: wake nodes, triangles, tip filaments and the trailing edge node of each wake node
  (src/wake/rigid.jl:53-62, built as rigid.jl:104-158).

Generators: ``icosphere`` (src/meshtools/bodies.jl:18-41), ``cube_sphere`` (bodies.jl:50-74) welded and split,
``scale_nodes`` (bodies.jl:103-108), node ``jitter`` and ``slivers`` (src/meshtools/abuse.jl:174-192, 339-360) with
this project's own seeded generator, and a rectangular NACA 00xx wing with ladder caps (the shape of
validation/common/reference_wing.jl, the quad split of src/geometry/quadsplit.jl and the cap ladder of
src/geometry/cap.jl) with its trailing-edge DOF map (src/dofmap/build.jl:118-316 for tip_kutta = :zero).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np
import scipy.sparse as sp


# --------------------------------------------------------------------------------------------------------------------
# data carried to the hot path


@dataclass
class Geometry:
    x: np.ndarray                      # (nnode, 3) float64
    tris: np.ndarray                   # (ntri, 3) int32, 0-based
    touch_pairs: np.ndarray = field(default_factory=lambda: np.zeros((0, 2), np.int32))
    name: str = ""

    @property
    def nnode(self) -> int:
        return self.x.shape[0]

    @property
    def ntri(self) -> int:
        return self.tris.shape[0]


@dataclass
class WakeTE:
    node: np.ndarray                   # body node of each wake trailing edge node
    x: np.ndarray                      # (nte, 3)
    lines: list                        # list of int arrays (indices into node)
    closed: list                       # bool per line


@dataclass
class DOFMapping:
    nslot: int
    nq: int
    corner_slot: np.ndarray            # (ntri, 3) int32
    C: sp.csr_matrix                   # nslot x nq
    K: sp.csr_matrix                   # nte x nq
    wake_te: WakeTE
    slot_area: np.ndarray
    slot_body: np.ndarray              # 1-based body of each slot (0: none)
    body_q: list                       # unknowns of each body (0-based)
    body_closed: list
    free_slot: np.ndarray              # slot of each unknown

    @property
    def q_body(self) -> np.ndarray:
        """1-based body of every unknown"""
        qb = np.zeros(self.nq, np.int32)
        for b, qs in enumerate(self.body_q):
            qb[np.asarray(qs, dtype=np.int64)] = b + 1
        return qb


@dataclass
class RigidWake:
    x: np.ndarray                      # (nw, 3)
    te: np.ndarray                     # wake trailing edge node of each wake node
    row: np.ndarray
    tris: np.ndarray                   # (nwtri, 3) int32
    filaments: np.ndarray              # (nfil, 2) int32
    rows: np.ndarray
    span: float

    @property
    def nwake(self) -> int:
        return self.x.shape[0]


def wake_rows(dm: DOFMapping, te_of_wake_node: np.ndarray) -> sp.csr_matrix:
    """Rows of the constraint matrix for the wake nodes: K[te, :] (src/dofmap/system.jl:132)"""
    return dm.K[np.asarray(te_of_wake_node, dtype=np.int64), :].tocsr()


# --------------------------------------------------------------------------------------------------------------------
# small geometry helpers


def _normalize(v):
    n = np.linalg.norm(v, axis=-1, keepdims=True)
    return v / np.where(n > 0, n, 1.0)


def tri_normals(x, tris):
    a, b, c = x[tris[:, 0]], x[tris[:, 1]], x[tris[:, 2]]
    return np.cross(b - a, c - a)


def slot_areas(x, tris, corner_slot, nslot):
    a = 0.5 * np.linalg.norm(tri_normals(x, tris), axis=1) / 3.0
    out = np.zeros(nslot)
    for k in range(3):
        np.add.at(out, corner_slot[:, k], a)
    return out


def closed_body_dofmap(g: Geometry) -> DOFMapping:
    """DOF map of closed, watertight, non-lifting bodies: one slot per node, every slot an unknown, one body
    (src/dofmap/build.jl:273-316 with no trailing edge, T-junction or gap)"""
    n = g.nnode
    C = sp.identity(n, format="csr")
    K = sp.csr_matrix((0, n))
    cs = g.tris.astype(np.int32).copy()
    area = slot_areas(g.x, g.tris, cs, n)
    te = WakeTE(np.zeros(0, np.int32), np.zeros((0, 3)), [], [])
    return DOFMapping(n, n, cs, C, K, te, area, np.ones(n, np.int32), [np.arange(n)], [True], np.arange(n))


# --------------------------------------------------------------------------------------------------------------------
# closed bodies


def icosphere(level: int, r: float = 1.0, center=(0.0, 0.0, 0.0)) -> Geometry:
    """Icosahedron subdivided ``level`` times, new nodes pushed onto the sphere (bodies.jl:18-41)"""
    phi = (1 + math.sqrt(5)) / 2
    P = [(-1.0, phi, 0), (1.0, phi, 0), (-1.0, -phi, 0), (1.0, -phi, 0), (0.0, -1, phi), (0.0, 1, phi),
         (0.0, -1, -phi), (0.0, 1, -phi), (phi, 0, -1), (phi, 0, 1), (-phi, 0, -1), (-phi, 0, 1)]
    P = [np.asarray(p, float) / np.linalg.norm(p) for p in P]
    F = [(1, 12, 6), (1, 6, 2), (1, 2, 8), (1, 8, 11), (1, 11, 12), (2, 6, 10), (6, 12, 5), (12, 11, 3), (11, 8, 7),
         (8, 2, 9), (4, 10, 5), (4, 5, 3), (4, 3, 7), (4, 7, 9), (4, 9, 10), (5, 10, 6), (3, 5, 12), (7, 3, 11),
         (9, 7, 8), (10, 9, 2)]
    F = [(a - 1, b - 1, c - 1) for a, b, c in F]
    for _ in range(level):
        mid = {}

        def m(a, b):
            key = (min(a, b), max(a, b))
            if key not in mid:
                p = P[a] + P[b]
                P.append(p / np.linalg.norm(p))
                mid[key] = len(P) - 1
            return mid[key]

        G = []
        for a, b, c in F:
            ab = m(a, b)
            bc = m(b, c)
            ca = m(c, a)
            G += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = G
    c0 = np.asarray(center, float)
    X = r * np.array(P) + c0
    T = np.array(F, dtype=np.int32)
    n = tri_normals(X, T)
    out = np.einsum("ij,ij->i", n, X[T].mean(axis=1) - c0)
    T[out < 0] = T[out < 0][:, ::-1]
    return Geometry(X, T, name=f"icosphere({level})")


def _weld(X, faces, rel=1e-3):
    """Merge nodes closer than rel times the shortest edge (the weld step of src/geometry/weld.jl)"""
    e = []
    for f in faces:
        m = len(f)
        for k in range(m):
            e.append(np.linalg.norm(X[f[k]] - X[f[(k + 1) % m]]))
    tol = rel * min(e)
    q = np.round(X / tol).astype(np.int64)
    keys = {}
    remap = np.empty(len(X), np.int64)
    newX = []
    for i, key in enumerate(map(tuple, q)):
        hit = None
        for dx in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dz in (-1, 0, 1):
                    kk = (key[0] + dx, key[1] + dy, key[2] + dz)
                    if kk in keys and np.linalg.norm(newX[keys[kk]] - X[i]) <= tol:
                        hit = keys[kk]
                        break
                if hit is not None:
                    break
            if hit is not None:
                break
        if hit is None:
            newX.append(X[i])
            hit = len(newX) - 1
            keys[key] = hit
        remap[i] = hit
    return np.array(newX), [[int(remap[v]) for v in f] for f in faces]


def _fold_angle(a, b, c, d):
    n1 = np.cross(b - a, c - a)
    n2 = np.cross(c - a, d - a)
    m = np.linalg.norm(n1) * np.linalg.norm(n2)
    if m <= 0:
        return 0.0
    return math.acos(max(-1.0, min(1.0, float(np.dot(n1, n2) / m))))


def _choose_diagonal(X, q, fold_deg=1.0, tie=1e-6, mirror=(1, 0.0)):
    """Diagonal of quad q (0: a-c, 1: b-d), following the rules of choose_diagonal (src/geometry/quadsplit.jl)"""
    a, b, c, d = X[q[0]], X[q[1]], X[q[2]], X[q[3]]
    L13, L24 = np.linalg.norm(c - a), np.linalg.norm(d - b)
    f13, f24 = _fold_angle(a, b, c, d), _fold_angle(b, c, d, a)
    if max(f13, f24) > math.radians(fold_deg) and abs(f13 - f24) > tie:
        return 0 if f13 < f24 else 1
    if abs(L13 - L24) > tie * max(L13, L24):
        return 0 if L13 < L24 else 1
    if mirror is not None:
        m, m0 = mirror
        centre = (a + b + c + d) / 4
        size = max(L13, L24)
        offset = centre[m] - m0
        if abs(offset) > tie * size:
            lo = np.minimum.reduce([a, b, c, d])
            hi = np.maximum.reduce([a, b, c, d])
            others = [k for k in range(3) if k != m]
            p = others[0] if hi[others[0]] - lo[others[0]] >= hi[others[1]] - lo[others[1]] else others[1]
            v13, v24 = c - a, d - b
            k13 = v13[m] * v13[p] * offset
            k24 = v24[m] * v24[p] * offset
            if abs(k13 - k24) > tie * size * size * abs(offset):
                return 0 if k13 > k24 else 1
    return 0 if min(q[0], q[2]) < min(q[1], q[3]) else 1


def split_quads(X, faces):
    tris = []
    for f in faces:
        if len(f) == 3:
            tris.append(tuple(f))
            continue
        a, b, c, d = f
        if _choose_diagonal(X, f) == 0:
            tris += [(a, b, c), (a, c, d)]
        else:
            tris += [(a, b, d), (b, c, d)]
    return np.array(tris, dtype=np.int32)


def _cube_sphere_faces(n: int, r: float = 1.0):
    X, quads = [], []
    for axis in range(3):
        for s in (-1.0, 1.0):
            a, b = [k for k in range(3) if k != axis]
            base = len(X)
            xi = [math.tan(math.pi / 4 * (2 * i / n - 1)) for i in range(n + 1)]
            for j in range(n + 1):
                for i in range(n + 1):
                    p = np.zeros(3)
                    p[axis] = s
                    p[a] = xi[i]
                    p[b] = xi[j]
                    X.append(r * p / np.linalg.norm(p))
            X_arr = X
            for j in range(n):
                for i in range(n):
                    f = [base + j * (n + 1) + i, base + j * (n + 1) + i + 1, base + (j + 1) * (n + 1) + i + 1,
                         base + (j + 1) * (n + 1) + i]
                    P = np.array([X_arr[v] for v in f])
                    nn = np.cross(P[1] - P[0], P[2] - P[0]) + np.cross(P[2] - P[0], P[3] - P[0])
                    if np.dot(nn, P.mean(axis=0)) < 0:
                        f = f[::-1]
                    quads.append(f)
    return np.array(X), quads


def cube_sphere(n: int, r: float = 1.0, split: bool = True):
    """Sphere of quads from an n x n equiangular grid per cube face (bodies.jl:50-74), welded; split into
    triangles when ``split`` (else the welded quads are returned as (X, faces))"""
    X, quads = _cube_sphere_faces(n, r)
    X, quads = _weld(X, quads)
    if not split:
        return X, quads
    return Geometry(X, split_quads(X, quads), name=f"cube_sphere({n})")


def scale_nodes(g, s):
    """Copy with node coordinates scaled by the 3-vector (or scalar) s (bodies.jl:103-108)"""
    s = np.broadcast_to(np.asarray(s, float), (3,))
    if isinstance(g, Geometry):
        return Geometry(g.x * s, g.tris.copy(), g.touch_pairs.copy(), g.name)
    X, faces = g
    return X * s, [list(f) for f in faces]


def ellipsoid_projector(axes):
    """The point where the ray from the centre through p meets the ellipsoid (validation/common/exact_flows.jl:68)"""
    ax = np.asarray(axes, float)

    def project(p):
        return p / math.sqrt(float(np.sum((p / ax) ** 2)))

    return project


def _node_frames(X, faces):
    """Unit node normals (area weighted), and each node's clearance over the edges of its elements that do not touch
    it (abuse.jl node_frames)"""
    n = np.zeros_like(X)
    clear = np.full(len(X), np.inf)
    for f in faces:
        m = len(f)
        a = np.cross(X[f[1]] - X[f[0]], X[f[2]] - X[f[0]])
        if m == 4:
            a = a + np.cross(X[f[2]] - X[f[0]], X[f[3]] - X[f[0]])
        for k in range(m):
            v = f[k]
            n[v] += a
            for j in range(m):
                if j == k or (j + 1) % m == k:
                    continue
                p, q = X[f[j]], X[f[(j + 1) % m]]
                e = q - p
                t = min(max(float(np.dot(X[v] - p, e) / max(np.dot(e, e), 1e-300)), 0.0), 1.0)
                clear[v] = min(clear[v], float(np.linalg.norm(X[v] - (p + t * e))))
    return _normalize(n), clear


def abuse(X, faces, jitter=None, slivers=None, project=None, seed=1):
    """Seeded node jitter and slivers on a welded quad/triangle surface, in that order with one random stream
    (abuse.jl:369-390 restricted to jitter and slivers). ``jitter = delta`` moves every node tangentially by up to
    delta times its clearance (abuse.jl:174-192); ``slivers = (n, ratio)`` moves n nodes, no two in one element,
    along one of their edges to ``ratio`` of its length (abuse.jl:339-360). Moved nodes go back onto the surface
    through ``project``. The random stream is this project's (numpy PCG64), so meshes are not those of the
    reference's StableRNG streams."""
    rng = np.random.default_rng(seed)
    X = np.array(X, float)
    nel = [[] for _ in range(len(X))]
    for e, f in enumerate(faces):
        for v in f:
            nel[v].append(e)
    if jitter is not None:
        normals, clear = _node_frames(X, faces)
        Y = X.copy()
        for v in range(len(X)):
            if not nel[v]:
                continue
            nv = normals[v]
            t1 = np.cross(nv, [1.0, 0, 0]) if abs(nv[0]) < 0.9 else np.cross(nv, [0, 1.0, 0])
            t1 /= np.linalg.norm(t1)
            t2 = np.cross(nv, t1)
            th = 2 * math.pi * rng.random()
            p = X[v] + jitter * clear[v] * rng.random() * (math.cos(th) * t1 + math.sin(th) * t2)
            Y[v] = project(p) if project is not None else p
        X = Y
    if slivers is not None:
        nsl, ratio = slivers
        blocked = set()
        count = 0
        for v in rng.permutation(len(X)):
            if count == nsl:
                break
            if v in blocked or not nel[v]:
                continue
            nbrs = []
            for e in nel[v]:
                f = faces[e]
                i = f.index(v)
                for s in (-1, 1):
                    w = f[(i + s) % len(f)]
                    if w not in nbrs:
                        nbrs.append(w)
            w = nbrs[int(rng.integers(len(nbrs)))]
            q = X[w] + ratio * (X[v] - X[w])
            X[v] = project(q) if project is not None else q
            for e in nel[v]:
                blocked.update(faces[e])
            count += 1
    return X, faces


# --------------------------------------------------------------------------------------------------------------------
# the rectangular NACA 00xx wing


def naca00_half_thickness(xi, t):
    """Half thickness of the NACA 00xx section with a sharp trailing edge at x/c = xi
    (validation/common/reference_wing.jl:38-41)"""
    xi = np.clip(xi, 0.0, 1.0)
    return 5 * t * (0.2969 * np.sqrt(xi) - 0.1260 * xi - 0.3516 * xi**2 + 0.2843 * xi**3 - 0.1036 * xi**4)


def _ladder(X, A, B, tie=1e-6):
    """Triangles between two chains sharing their first and last nodes (src/geometry/cap.jl ladder)"""
    p, q = len(A) - 1, len(B) - 1

    def arclen(C):
        s = np.concatenate([[0.0], np.cumsum(np.linalg.norm(np.diff(X[C], axis=0), axis=1))])
        return s / s[-1]

    if p == 1 or q == 1:
        raise ValueError("cap chains need at least two segments each")
    sA, sB = arclen(A), arclen(B)
    tris = [(A[0], A[1], B[1])]
    i, j = 1, 1
    toggle = False
    while not (i == p - 1 and j == q - 1):
        if i == p - 1:
            adv_a = False
        elif j == q - 1:
            adv_a = True
        else:
            dA = np.linalg.norm(X[A[i + 1]] - X[B[j]])
            dB = np.linalg.norm(X[A[i]] - X[B[j + 1]])
            if abs(dA - dB) > tie * max(dA, dB):
                adv_a = dA < dB
            elif abs(sA[i + 1] - sB[j + 1]) > tie:
                adv_a = sA[i + 1] < sB[j + 1]
            else:
                toggle = not toggle
                adv_a = toggle
        if adv_a:
            tris.append((A[i], A[i + 1], B[j]))
            i += 1
        else:
            tris.append((A[i], B[j + 1], B[j]))
            j += 1
    tris.append((A[p - 1], A[p], B[q - 1]))
    return tris


@dataclass
class Wing:
    g: Geometry
    dm: DOFMapping
    span: float
    chord: float
    nchord: int
    nspan: int


def wing(nchord: int, nspan: int, aspect: float = 8.0, chord: float = 1.0, thickness: float = 0.12) -> Wing:
    """Rectangular, untwisted NACA 00xx wing (chord along +x from the leading edge at x = 0, span along y centred on
    y = 0, thickness along z), ``nchord`` full-cosine chordwise panels per side and ``nspan`` full-cosine spanwise
    panels, quads split into triangles, the tips closed by ladder caps, the sharp trailing edge shared by both surfaces.
    The DOF map duplicates every trailing edge node for the lower surface, ties the lower copies at the two tips to
    the upper ones (tip_kutta = :zero), and has one open wake trailing edge line along +y."""
    span = aspect * chord
    xi = (1 - np.cos(np.pi * np.arange(nchord + 1) / nchord)) / 2
    ys = span * (-0.5 + (1 - np.cos(np.pi * np.arange(nspan + 1) / nspan)) / 2)
    zt = chord * naca00_half_thickness(xi, thickness)
    zt[0] = 0.0
    zt[-1] = 0.0
    nc = nchord
    per = 2 * nc  # nodes per station: LE, upper 1..nc-1, TE, lower 1..nc-1

    def up(i, j):
        return j * per + i  # i = 0 (LE) .. nc (TE)

    def low(i, j):
        if i == 0:
            return j * per
        if i == nc:
            return j * per + nc
        return j * per + nc + i

    X = np.zeros(((nspan + 1) * per, 3))
    for j in range(nspan + 1):
        for i in range(nc + 1):
            X[up(i, j)] = (xi[i] * chord, ys[j], zt[i])
            X[low(i, j)] = (xi[i] * chord, ys[j], -zt[i])
    quads, side = [], []
    for j in range(nspan):
        for i in range(nc):
            quads.append([up(i, j), up(i + 1, j), up(i + 1, j + 1), up(i, j + 1)])
            side.append(1)
    for j in range(nspan):
        for i in range(nc):
            quads.append([low(i, j + 1), low(i + 1, j + 1), low(i + 1, j), low(i, j)])
            side.append(-1)
    tris, tside = [], []
    for f, s in zip(quads, side):
        a, b, c, d = f
        if _choose_diagonal(X, f) == 0:
            tris += [(a, b, c), (a, c, d)]
        else:
            tris += [(a, b, d), (b, c, d)]
        tside += [s, s]
    # caps: ladder between the upper (A) and lower (B) chains of each tip section, oriented outward (-y, +y)
    for j, out in ((0, -1.0), (nspan, 1.0)):
        A = [up(i, j) for i in range(nc + 1)]
        B = [low(i, j) for i in range(nc + 1)]
        for t in _ladder(X, A, B):
            nrm = np.cross(X[t[1]] - X[t[0]], X[t[2]] - X[t[0]])
            if nrm[1] * out < 0:
                t = (t[0], t[2], t[1])
            tris.append(t)
            tside.append(0)
    T = np.array(tris, dtype=np.int32)
    tside = np.array(tside)
    g = Geometry(X, T, name=f"wing AR{aspect:g} {nchord}x{nspan}")
    nn = len(X)
    # slots: lower copies of the trailing edge nodes (assign_slots, build.jl:118-147; caps take the upper copy)
    te_nodes = np.array([up(nc, j) for j in range(nspan + 1)], dtype=np.int64)
    lower_slot = np.full(nn, -1, np.int64)
    lower_slot[te_nodes] = nn + np.arange(nspan + 1)
    nslot = nn + nspan + 1
    cs = T.astype(np.int64).copy()
    for t in np.nonzero(tside == -1)[0]:
        for k in range(3):
            if lower_slot[cs[t, k]] >= 0:
                cs[t, k] = lower_slot[cs[t, k]]
    # tip_kutta = :zero: the lower copies at both tips are tied to the upper ones (tip_constraints!, build.jl:211-226)
    tied = {int(lower_slot[te_nodes[0]]): int(te_nodes[0]), int(lower_slot[te_nodes[-1]]): int(te_nodes[-1])}
    free = np.array([s for s in range(nslot) if s not in tied], dtype=np.int64)
    q_of_slot = np.full(nslot, -1, np.int64)
    q_of_slot[free] = np.arange(len(free))
    rows, cols = [], []
    for s in range(nslot):
        f = tied.get(s, s)
        rows.append(s)
        cols.append(q_of_slot[f])
    nq = len(free)
    C = sp.csr_matrix((np.ones(nslot), (rows, cols)), shape=(nslot, nq))
    # Kutta rows (wake_trailing_edge, kutta.jl:357-425): mu_w = mu_upper - mu_lower along the line, tau = +y
    nte = nspan + 1
    U = sp.csr_matrix((np.ones(nte), (np.arange(nte), te_nodes)), shape=(nte, nslot))
    L = sp.csr_matrix((np.ones(nte), (np.arange(nte), lower_slot[te_nodes])), shape=(nte, nslot))
    K = ((U - L) @ C).tocsr()
    K.eliminate_zeros()
    wte = WakeTE(te_nodes.astype(np.int32), X[te_nodes].copy(), [np.arange(nte)], [False])
    area = slot_areas(X, T, cs, nslot)
    dm = DOFMapping(nslot, nq, cs.astype(np.int32), C, K, wte, area, np.ones(nslot, np.int32), [np.arange(nq)],
                    [True], free)
    return Wing(g, dm, span, chord, nchord, nspan)


def te_panel_size(g: Geometry, dm: DOFMapping) -> float:
    """Median height of the trailing edge triangles over their trailing edge (rigid.jl:75-95)"""
    te = set(int(v) for v in dm.wake_te.node)
    h = []
    for t in g.tris:
        on = [v for v in t if int(v) in te]
        if len(on) == 2:
            c = [v for v in t if int(v) not in te][0]
            a, b = on
            h.append(np.linalg.norm(np.cross(g.x[b] - g.x[a], g.x[c] - g.x[a])) / np.linalg.norm(g.x[b] - g.x[a]))
    h.sort()
    return float(h[(len(h) + 1) // 2 - 1])


def build_wake(g: Geometry, dm: DOFMapping, direction, length: float = 20.0, first_row=None, growth: float = 1.2,
               rows=None, ending: str = "truncate") -> RigidWake:
    """Rigid wake strips from the wake trailing edge nodes along ``direction`` (build_wake, rigid.jl:104-158, with
    direction = :freestream taken along the given vector): rows at 0, l1, l1(1 + r), ... until ``length`` spans;
    ``ending = "closed"`` adds the far-end filament (the trailing edge panel of a free wake, te_panel)."""
    wte = dm.wake_te
    n = len(wte.node)
    if n == 0:
        raise ValueError("the geometry has no trailing edge to shed a wake from")
    d = np.asarray(direction, float)
    d = d / np.linalg.norm(d)
    span = float(max(np.linalg.norm(wte.x[i] - wte.x[j]) for i in range(n) for j in range(n)))
    if rows is None:
        l1 = te_panel_size(g, dm) if first_row is None else float(first_row)
        rows = [0.0, l1]
        while rows[-1] < length * span:
            rows.append(rows[-1] + (rows[-1] - rows[-2]) * growth)
    rows = np.asarray(rows, float)
    nrow = len(rows) - 1
    x = np.zeros((n * (nrow + 1), 3))
    for j in range(nrow + 1):
        x[j * n:(j + 1) * n] = wte.x + rows[j] * d
    te = np.tile(np.arange(n), nrow + 1)
    row = np.repeat(np.arange(nrow + 1), n)
    tris, fil = [], []

    def idx(k, j):
        return j * n + k

    for line, closed in zip(wte.lines, wte.closed):
        m = len(line)
        segs = [(line[i], line[i + 1]) for i in range(m - 1)]
        if closed:
            segs.append((line[m - 1], line[0]))
        for A, B in segs:
            for j in range(nrow):
                tris.append((idx(A, j), idx(A, j + 1), idx(B, j)))
                tris.append((idx(A, j + 1), idx(B, j + 1), idx(B, j)))
        if not closed:
            fil += [(idx(line[0], j + 1), idx(line[0], j)) for j in range(nrow)]
            fil += [(idx(line[m - 1], j), idx(line[m - 1], j + 1)) for j in range(nrow)]
        if ending == "closed":
            fil += [(idx(B, nrow), idx(A, nrow)) for A, B in segs]
    return RigidWake(x, te.astype(np.int32), row.astype(np.int32), np.array(tris, np.int32).reshape(-1, 3),
                     np.array(fil, np.int32).reshape(-1, 2), rows, span)


def te_panel(g: Geometry, dm: DOFMapping, direction, length=None) -> RigidWake:
    """The implicit trailing edge panel of a free wake: one row, closed by its downstream filament (rigid.jl:162-163)"""
    L = te_panel_size(g, dm) if length is None else float(length)
    return build_wake(g, dm, direction, rows=[0.0, L], ending="closed")


# --------------------------------------------------------------------------------------------------------------------
# the workloads


def sphere_case(level: int = 3):
    """Unit icosphere, closed-body DOF map"""
    g = icosphere(level)
    return g, closed_body_dofmap(g)


def ellipsoid_case(n: int = 32, axes=(3.0, 1.0, 1.0), jitter: float = 0.2, slivers=(10, 0.02), seed: int = 7):
    """cube_sphere(n) scaled to the ellipsoid, jittered and slivered with nodes projected back onto the surface"""
    X, faces = cube_sphere(n, split=False)
    X, faces = scale_nodes((X, faces), axes)
    proj = ellipsoid_projector(axes)
    X, faces = abuse(X, faces, jitter=jitter, slivers=slivers, project=proj, seed=seed)
    g = Geometry(X, split_quads(X, faces), name=f"ellipsoid {axes} cube_sphere({n}) abused")
    return g, closed_body_dofmap(g)
