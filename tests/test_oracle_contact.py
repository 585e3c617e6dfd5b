"""The oracle's touching and contact tiers (src/assembly/assemble.jl:102-238) after the reference's
test/assembly/test_contact.jl: the pieces of the contact rule at a T-junction, a reversed pair and a point contact,
and the pair blocks of the contact, wide-corner and several-contact rules against cubature over the test triangle.

The referee integrates the same closed-form kernel (restated here in numpy) over (u, v) -> λ = (1-u, u(1-v), uv),
dA = 2A u du dv, with tensor tanh-sinh rules, whose nodes cluster at the ends where these singularities sit, split
at the end of a singular segment. It converges to ~1e-12 between levels 6 and 8 on every case below. It agrees with
scipy's adaptive quad_vec (nested, epsrel 1e-9) to 1e-11 on the T-junction block, and to 4e-13 on the 0.1% gap and
the needle."""
import math

import numpy as np
import pytest

TA, TB, TH = np.array([0.0, 0.0, 0.0]), np.array([1.0, 0.0, 0.0]), np.array([0.5, 0.0, 0.0])
# a T-junction: T's long edge a-b with the hanging node h at its middle; S = (h, a, c) across it, folded by 20°
TLONG = np.array([TA, TB, [0.45, -0.8, 0.0]])
TSHORT = np.array([TH, TA, [0.2, 0.7 * math.cos(math.radians(20)), 0.7 * math.sin(math.radians(20))]])


def _dir(deg):
    return np.array([math.cos(math.radians(deg)), math.sin(math.radians(deg)), 0.0])


def _shared(T, S):
    return tuple(int(any(np.array_equal(t, s) for s in S)) for t in T)


def _mono(a, b, c):
    return 2 * math.factorial(a) * math.factorial(b) * math.factorial(c) / math.factorial(a + b + c + 2)


def _w_exact(S, x):
    """the unit source triangle's velocity (source_triangle.jl:75-89) at points x (n x 3), FP64"""
    n = np.cross(S[1] - S[0], S[2] - S[0])
    n /= np.linalg.norm(n)
    R = [x - S[k] for k in range(3)]
    L = [np.sqrt((r * r).sum(-1)) for r in R]
    wt = np.zeros_like(x)
    for e in range(3):
        i, j = e, (e + 1) % 3
        d = np.linalg.norm(S[j] - S[i])
        nu = np.cross(S[j] - S[i], n)
        nu /= np.linalg.norm(nu)
        p = (R[i] * R[j]).sum(-1)
        num = L[i] + L[j] + d
        c2 = (np.cross(R[i], R[j]) ** 2).sum(-1)
        with np.errstate(divide="ignore", invalid="ignore"):
            plus = np.log(num * num / (2 * (L[i] * L[j] + p)))
            minus = np.log(num * num * ((L[i] * L[j] - p) / (2 * c2)))  # cancellation-free where p < 0
        wt += np.where(p >= 0, plus, minus)[:, None] * nu
    N = (R[0] * np.cross(R[1], R[2])).sum(-1)
    D = L[0] * L[1] * L[2] + (R[0] * R[1]).sum(-1) * L[2] + (R[0] * R[2]).sum(-1) * L[1] + (R[1] * R[2]).sum(-1) * L[0]
    return (wt + 2 * np.arctan2(N, D)[:, None] * n) / (4 * math.pi)


def _tanh_sinh(a, b, level):
    h = 2.0 ** -level
    t = np.arange(-int(6 / h), int(6 / h) + 1) * h
    s = 0.5 * math.pi * np.sinh(t)
    x = np.tanh(s)
    w = h * 0.5 * math.pi * np.cosh(t) / np.cosh(s) ** 2
    keep = (np.abs(x) < 1) & (w > 1e-300)
    x, w = x[keep], w[keep]
    d = (b - a) / 2
    return np.where(x < 0, a + d * (1 + x), b - d * (1 - x)), w * d  # distances to the ends kept accurate


def block_cubature(T, S, ubreaks=(), level=6):
    """∫ψ_a n_T·(γ_b × w_S) dA over T, hat ψ (the 3 x 3 block of pair_block, assemble.jl:245-258)"""
    nA = np.cross(T[1] - T[0], T[2] - T[0])
    AT = np.linalg.norm(nA) / 2
    nT = nA / (2 * AT)
    SA2 = np.linalg.norm(np.cross(S[1] - S[0], S[2] - S[0]))
    gS = [-(S[2] - S[1]) / SA2, -(S[0] - S[2]) / SA2, -(S[1] - S[0]) / SA2]
    v, wv = _tanh_sinh(0.0, 1.0, level)
    br = [0.0, *ubreaks, 1.0]
    out = np.zeros(9)
    for k in range(len(br) - 1):
        u, wu = _tanh_sinh(br[k], br[k + 1], level)
        U, V = (a.ravel() for a in np.meshgrid(u, v, indexing="ij"))
        W = np.outer(wu, wv).ravel()
        lam = np.stack([1 - U, U * (1 - V), U * V], axis=1)
        wn = np.cross(_w_exact(S, lam @ T), nT)
        g = np.stack([wn @ gS[0], wn @ gS[1], wn @ gS[2]], axis=1)
        out += ((lam[:, :, None] * g[:, None, :]).reshape(-1, 9) * (W * 2 * AT * U)[:, None]).sum(0)
    return out.reshape(3, 3)


def _err(oracle, T, S, lam, w, ref):
    blk, _ = oracle.pair_block(T, S, lam, w, kernel_far=math.inf)
    return np.linalg.norm(blk - ref) / np.linalg.norm(ref)


@pytest.fixture(scope="module")
def sizes(oracle):
    return {k: len(oracle.rule(k)[1]) for k in ("edge", "vertex", "self")}


def test_contact_pieces(oracle, sizes):
    tier, lam, w = oracle.pair_rule(TLONG, TSHORT, shared=_shared(TLONG, TSHORT))
    # split at h: the piece along a-h carries the edge rule, the piece h-b-c the corner rule toward h, in two parts
    # as that corner is 94° wide
    assert tier == "contact" and len(w) == sizes["edge"] + 2 * sizes["vertex"]
    assert abs(w.sum() - 1) < 1e-13
    assert np.all(lam >= -1e-15) and np.abs(lam.sum(1) - 1).max() < 1e-14
    for p, q, s in ((1, 0, 0), (2, 1, 0), (1, 1, 1), (3, 0, 2)):
        got = float(w @ (lam[:, 0] ** p * lam[:, 1] ** q * lam[:, 2] ** s))
        assert abs(got / _mono(p, q, s) - 1) < 1e-12
    # the reverse pair: S's whole edge h-a lies on T's long edge, so T takes the edge rule unsplit
    tier, _, w = oracle.pair_rule(TSHORT, TLONG, shared=_shared(TSHORT, TLONG))
    assert tier == "contact" and len(w) == sizes["edge"]
    # a point contact at the hanging node: both pieces carry the corner rule toward h, the 94° one in two parts
    S = np.array([TH, [0.3, 0.5, 0.1], [0.7, 0.5, 0.1]])
    tier, _, w = oracle.pair_rule(TLONG, S, shared=_shared(TLONG, S))
    assert tier == "contact" and len(w) == 3 * sizes["vertex"]
    # regular neighbours (a shared edge, a shared corner) and a distant triangle take no contact rule
    for S, want in ((np.array([TB, TA, [0.4, 0.7, 0.2]]), "edge"), (np.array([TB, [1.6, 0.4, 0.0], [1.2, 0.8, 0.1]]), "vertex"),
                    (np.array([[0.0, 0.0, 2.0], [1.0, 0.0, 2.0], [0.5, 1.0, 2.0]]), None)):
        tier, _, _ = oracle.pair_rule(TLONG, S, shared=_shared(TLONG, S))
        assert tier != "contact" and (want is None or tier == want)


def test_contact_accuracy(oracle):
    for T, S, br in ((TLONG, TSHORT, (0.5,)), (TSHORT, TLONG, ())):
        ref = block_cubature(T, S, br)
        _, lam, w = oracle.pair_rule(T, S, shared=_shared(T, S))
        assert _err(oracle, T, S, lam, w, ref) < 1e-6
        # the rule of the shared corner alone misses the singular segment
        k = _shared(T, S).index(1)
        lam, w = oracle.rule("vertex", k=k)
        assert _err(oracle, T, S, lam, w, ref) > 1e-3
    # a gap: S faces T's edge a-b across a slit of 1% and 0.1% of its length, sharing no node. The graded edge rule
    # resolves the near singularity whatever the width; the distance tiers alone would take the near rule
    for gap in (0.01, 0.001):
        S = np.array([TB + [0, gap, 0], TA + [0, gap, 0], [0.5, 0.7, 0.3]])
        ref = block_cubature(TLONG, S)
        tier, lam, w = oracle.pair_rule(TLONG, S)
        assert tier == "contact" and _err(oracle, TLONG, S, lam, w, ref) < 1e-6
        tier, lam, w = oracle.pair_rule(TLONG, S, contact_rel=1e-12)
        assert tier == "near" and _err(oracle, TLONG, S, lam, w, ref) > 1e-4


def test_wide_corners(oracle, sizes):
    # T's corner at the origin is 150° wide and S shares it beyond a 20° gap: in two equal angles the vertex rule is
    # as accurate as on a narrow corner, while the stored rule under-samples the middle of the corner
    T = np.array([TA, _dir(-75), _dir(75)])
    S = np.array([TA, 0.9 * _dir(95) + [0, 0, 0.1], 1.1 * _dir(145) + [0, 0, 0.2]])
    ref = block_cubature(T, S)
    tier, lam, w = oracle.pair_rule(T, S, shared=_shared(T, S))
    assert tier == "vertex" and len(w) == 2 * sizes["vertex"] and abs(w.sum() - 1) < 1e-13
    assert _err(oracle, T, S, lam, w, ref) < 1e-7
    lam, w = oracle.rule("vertex")
    assert _err(oracle, T, S, lam, w, ref) > 1e-4
    # corners up to 90° keep the stored rule; 170° takes three pieces (vertex_rule alone: a source sharing the corner
    # only, with the contact test's tolerance at zero, as the 170° corner lies within it of T's opposite edge)
    S = np.array([TA, 0.9 * _dir(175) + [0, 0, 0.3], 0.9 * _dir(-175) + [0, 0, 0.3]])
    for half, pieces in ((45, 1), (85, 3)):
        T = np.array([TA, _dir(-half), _dir(half)])
        tier, _, w = oracle.pair_rule(T, S, shared=_shared(T, S), contact_rel=1e-12)
        assert tier == "vertex" and len(w) == pieces * sizes["vertex"]


def test_several_contacts(oracle, sizes):
    # a needle sharing S's corner a and lying along S's edge a-b, its other corners within the tolerance of that
    # edge: no single edge or corner of T carries the singular set, so T takes the self rule
    S = np.array([TA, TB, [0.5, 0.8, 0.0]])
    T = np.array([TA, [0.3, -0.05, 0.0], [0.6, -0.03, 0.0]])
    tier, lam, w = oracle.pair_rule(T, S, shared=_shared(T, S))
    assert tier == "contact" and len(w) == sizes["self"]
    assert _err(oracle, T, S, lam, w, block_cubature(T, S)) < 1e-6
