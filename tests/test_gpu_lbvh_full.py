"""Standalone broad phase at full size: 2^20 random triangles, 2^20 vertex
queries with padding 2e-3.  Codes, sort order and topology are compared with the
oracle bit for bit; candidate lists on a sample of queries; size-independent
properties on all of them."""
import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

N = 1 << 20


@pytest.fixture(scope="module")
def soup(pkg, po):
    verts, faces, queries = pkg.scenes.triangle_soup(N, seed=0)
    V4 = np.zeros((verts.shape[0], 4), np.float32)
    V4[:, :3] = verts
    Q4 = np.zeros((N, 4), np.float32)
    Q4[:, :3] = queries
    mn, mx = po.face_aabbs(V4, faces, 0.0)
    box = po.scene_aabb(V4, 0.0)
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    bvh = pkg.LBVH(N, "cuda", tie=1)
    bvh.build(t(mn), t(mx), t(box))
    cand, num = bvh.query(t(Q4), 2e-3, 32)
    torch.cuda.synchronize()
    return dict(mn=mn, mx=mx, box=box, Q4=Q4, bvh=bvh, cand=cand.cpu().numpy(), num=num.cpu().numpy())


def test_full_size_matches_oracle(po, soup):
    ref = po.FaceBVH(soup["mn"], soup["mx"], soup["box"], tie=1)
    b = soup["bvh"]
    assert np.array_equal(b.codes.cpu().numpy(), ref.sorted_codes)
    assert np.array_equal(b.sorted_ids.cpu().numpy(), ref.sorted_ids)
    for name in ("child_a", "child_b", "range_l", "range_r", "parent"):
        assert np.array_equal(getattr(b, name).cpu().numpy(), getattr(ref, name)), name
    assert np.array_equal(b.node_min4.cpu().numpy(), ref.nmin4)
    assert np.array_equal(b.node_max4.cpu().numpy(), ref.nmax4)
    sample = np.arange(0, N, 97)
    qmn, qmx = po.query_boxes(soup["Q4"][sample], 2e-3)
    rc, rn, _ = ref.traverse(qmn, qmx, 32)
    assert np.array_equal(soup["num"][sample], rn)
    for i, q in enumerate(sample):
        k = min(rn[i], 32)
        assert np.array_equal(soup["cand"][q, :k], rc[i, :k])


def test_full_size_properties(soup):
    b = soup["bvh"]
    codes = b.codes.cpu().numpy().view(np.uint32)
    ids = b.sorted_ids.cpu().numpy()
    assert np.all(codes[1:] >= codes[:-1])
    assert np.array_equal(np.sort(ids), np.arange(N))
    ca, cb = b.child_a.cpu().numpy(), b.child_b.cpu().numpy()
    kids = np.concatenate([ca, cb])
    assert np.array_equal(np.sort(kids), np.arange(1, 2 * N - 1))   # every node but the root has one parent
    # each query is a vertex of its own triangle: that triangle is always a candidate
    num, cand = soup["num"], soup["cand"]
    ok = num <= 32
    own = (cand == np.arange(N)[:, None]).any(axis=1)
    assert np.all(own[ok])
    assert num.min() >= 1


def test_full_size_reference_tie_rule(pkg, po, soup):
    """The same 2^20 soup under the reference's equal-code rule (tie = 0:
    delta = 32 for equal codes, lbvh_cell.py:256-264): codes, sort order and
    the child and range arrays equal the oracle's bit for bit at full size.
    The soup has repeated codes, so the tree is the reference's malformed one;
    parents are compared where a node is claimed by exactly one internal node
    (a node claimed twice gets the last serial writer in the oracle and a
    racing writer on the GPU)."""
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a)).cuda()  # noqa: E731
    bvh = pkg.LBVH(N, "cuda", tie=0)
    bvh.build(t(soup["mn"]), t(soup["mx"]), t(soup["box"]))
    torch.cuda.synchronize()
    ref = po.FaceBVH(soup["mn"], soup["mx"], soup["box"], tie=0)
    codes = bvh.codes.cpu().numpy()
    assert np.array_equal(codes, ref.sorted_codes)
    assert len(np.unique(codes)) < N   # repeated codes: the tie rule matters
    assert np.array_equal(bvh.sorted_ids.cpu().numpy(), ref.sorted_ids)
    for name in ("child_a", "child_b", "range_l", "range_r"):
        assert np.array_equal(getattr(bvh, name).cpu().numpy()[: N - 1], getattr(ref, name)[: N - 1]), name
    kids = np.concatenate([ref.child_a[: N - 1], ref.child_b[: N - 1]])
    once = np.bincount(kids, minlength=2 * N - 1) == 1
    assert np.array_equal(bvh.parent.cpu().numpy()[once], ref.parent[once])
