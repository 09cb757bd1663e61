"""CPU: the traversal oracle (oracle/dda.c) against fixtures produced by the
reference's own CUDA kernels (tests/golden/traverse_ref.npz, made by
tests/golden/make_traverse_golden.py).  Bit-exact."""
import numpy as np
import pytest

from oracle import native as orc


def unpack(bits, n):
    return np.unpackbits(bits)[: n ** 3].reshape(n, n, n).astype(bool)


def maxpool(m, s):
    n = m.shape[0] // s
    return m.reshape(n, s, n, s, n, s).any(axis=(1, 3, 5))


def same_bits(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


@pytest.fixture(scope="module")
def g(golden):
    return golden("traverse_ref.npz")


def test_dense_walk_matches_reference_kernel(g):
    n = int(g["walk_n"])
    inter, num, tns = orc.dense_walk(g["walk_o"], g["walk_v"], float(g["walk_xyzmin"]), n, float(g["walk_vs"]))
    assert np.array_equal(num, g["dense_num"])
    assert same_bits(orc.csr_from_padded(inter, num), g["dense_pts"])
    assert same_bits(orc.csr_from_padded(tns[..., None], num)[:, 0], g["dense_tns"])
    assert same_bits(inter[:, 0], g["dense_row0"])


@pytest.mark.parametrize("tag,scale", [("m1", 1.0), ("m05", 0.5), ("m025", 0.25)])
def test_masked_walk_matches_reference_kernel(g, tag, scale):
    n = int(g["walk_n"])
    m = unpack(g["mask64"], n)
    if scale != 1.0:
        m = maxpool(m, int(round(1 / scale)))
    inter, num, tns = orc.masked_walk(g["walk_o"], g["walk_v"], float(g["walk_xyzmin"]), n, float(g["walk_vs"]), m, scale)
    assert np.array_equal(num, g[f"masked_{tag}_num"])
    assert same_bits(orc.csr_from_padded(inter, num), g[f"masked_{tag}_seg"])
    assert same_bits(orc.csr_from_padded(tns[..., None], num)[:, 0], g[f"masked_{tag}_tns"])


def octree_march_oracle(g, N, fused=True):
    m = unpack(g[f"oct{N}_mask"], N)
    octs = np.concatenate([maxpool(m, s).reshape(-1) for s in (64, 16, 4)])
    v = g[f"oct{N}_v"]
    B = v.shape[0]
    coords = np.zeros((8, B, 6), np.float32)
    rgba = np.zeros((B, 4), np.float32)
    finish = np.zeros(B, np.uint8)
    orc.aabb(coords, v, g[f"oct{N}_center"], finish, rgba, octs, N, fused)
    resume = coords[7, :, 3:].copy()
    fin0 = finish.copy()
    hits = [[] for _ in range(B)]
    rounds = 0
    while not finish.all() and rounds < 4 * N:
        active = finish == 0
        orc.ray_march(coords, v, m, finish, N, fused)
        for b in np.nonzero(active)[0]:
            for h in range(8):
                if coords[h, b, 0] < 0:
                    break
                hits[b].append(coords[h, b].copy())
        finish |= (coords[:, :, 0] < 0).any(0).astype(np.uint8)
        rounds += 1
    return resume, fin0, rgba, hits, rounds


@pytest.mark.parametrize("N", [128, 256])
def test_octree_and_march_match_reference_kernels(g, N):
    resume, fin0, rgba, hits, rounds = octree_march_oracle(g, N)
    ref_fin = g[f"oct{N}_finish"].astype(bool)
    assert np.array_equal(fin0.astype(bool), ref_fin)
    live = ~ref_fin
    assert same_bits(resume[live], g[f"oct{N}_resume"][live])
    assert same_bits(rgba, g[f"oct{N}_rgba"])
    num = np.array([len(h) for h in hits], np.int32)
    assert np.array_equal(num, g[f"oct{N}_hit_num"])
    flat = np.concatenate([np.asarray(h, np.float32).reshape(-1, 6) for h in hits], 0)
    assert same_bits(flat, g[f"oct{N}_hits"])
    assert rounds == int(g[f"oct{N}_rounds"])


def test_fixture_exercises_edge_cases(g):
    # the fixture holds misses, rays starting inside, and long rays
    num = g["dense_num"]
    assert (num == 0).any() and (num > 100).any()
    assert (g[f"masked_m1_num"] == 0).any()
    assert g["oct128_finish"].any() and not g["oct128_finish"].all()


def test_unfused_position_update_differs_from_reference(g):
    """The reference's compiler contracts ori + dir*t into one fused multiply-add:
    the same walk with a separately rounded product diverges from the fixture."""
    n = int(g["walk_n"])
    inter, num, tns = orc.dense_walk(g["walk_o"], g["walk_v"], float(g["walk_xyzmin"]), n, float(g["walk_vs"]), fused=False)
    pts = orc.csr_from_padded(inter, num)
    assert not (np.array_equal(num, g["dense_num"]) and same_bits(pts, g["dense_pts"]))
