"""The engine against the reference's own GPU build, through the C ABI.

tests/golden/ref_gpu_golden.npz holds outputs of the reference's CUDA code
(z_norm_gpu_x, idx_init, NCC_3D + get_pos_idx, extract_shape, k_shape /
k_shape_tsl with the driver's restart), compiled for sm_103a from the
reference's headers and run on a GB300 by tests/golden/make_ref_gpu_golden.py,
with the inputs stored beside them.  Every case here uses compat FFT lengths
that wrap (F < 2m - 1); m = 100 and 129 also take get_pos_idx's pad-with-2.

What is compared (compat mode, FP32 form):
* initial labels of init_chose=0: identical;
* assignment: labels identical, distances within 2e-6;
* z-norm: within 2e-6;
* extraction: counts and non-empty cluster numbers identical, centroids within
  1e-5 relative (max |c - c_ref| <= 1e-5 max |c_ref|), for zero starts (gate
  closed), raw-row starts (gate open: members aligned) and unit-norm starts,
  cal_select 0 (m power steps) and 1 (the syevd path);
* the whole loop (init_chose 0, and 1 with mt19937 seeds 0 and 1): labels,
  non-empty cluster count and restart flag identical.

The reference's z-norm reads one shared-memory slot it never writes when
m < 1024 (Code/include/normalization.cuh:36-39 writes sh_row[tid] only for
tid < m and tid > m).  On the GB300 that slot held non-zero data at m = 100 and
m = 128: a quarter of the rows came out mis-scaled and some NaN (the stored
znorm outputs show it).  The assignment is scale-invariant, so it is compared
at those lengths too; z-norm, extraction and the loop, which depend on those
scales, are compared at m = 129, 300 and 512, where the slot held zero.
"""
import hashlib
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.environ.get("TIMESC_REF_GOLDEN", os.path.join(HERE, "golden", "ref_gpu_golden.npz"))
GOLDEN_C2 = os.environ.get("TIMESC_REF_GOLDEN_C2", os.path.join(HERE, "golden", "ref_gpu_c2.npz"))
CASES = ["c1", "w100", "w129", "w300", "w512"]
CLEAN = ["w129", "w300", "w512"]  # the reference's z-norm read a zero slot


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


def _meta(g, name):
    n, m, k, cap = (int(v) for v in g[name + "__meta"])
    return n, m, k, cap


def _cuda(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(a)).cuda()


@pytest.mark.parametrize("name", CASES)
def test_init_labels_match_reference(built, gpu_ctx, gold, name):
    import torch
    n, m, k, _ = _meta(gold, name)
    lab = torch.full((n,), -1, dtype=torch.int32, device="cuda")
    gpu_ctx.init_labels(lab, k)
    assert np.array_equal(lab.cpu().numpy() + 1, gold[name + "__init"])


@pytest.mark.parametrize("name", CASES)
@pytest.mark.parametrize("cents", ["ext", "raw"])
def test_assign_matches_reference(built, gpu_ctx, gold, name, cents):
    import torch
    T, _ = built
    n, m, k, _ = _meta(gold, name)
    xz = gold[name + "__xz"]
    C = gold[name + "__extract_zero_cal0__centroids"] if cents == "ext" else gold[name + "__x"][gold[name + "__raw_rows"]]
    lab = torch.zeros(n, dtype=torch.int32, device="cuda")
    dist = torch.zeros(n, dtype=torch.float32, device="cuda")
    gpu_ctx.sbd_assign(_cuda(xz), _cuda(C.astype(np.float32)), mode=T.MODE_COMPAT, precision=T.PREC_FP32,
                       labels=lab, dist=dist)
    L, D = lab.cpu().numpy(), dist.cpu().numpy()
    Lr, Dr = gold["%s__assign_%s__labels" % (name, cents)] - 1, gold["%s__assign_%s__dist" % (name, cents)]
    derr = float(np.abs(D - Dr).max())
    print("assign %s/%s: labels differ %d of %d, max |d - d_ref| %.2e" % (name, cents, int((L != Lr).sum()), n, derr))
    assert np.array_equal(L, Lr)
    assert derr <= 2e-6


@pytest.mark.parametrize("name", CLEAN)
def test_znorm_matches_reference(built, gpu_ctx, gold, name):
    x = _cuda(gold[name + "__x"])
    gpu_ctx.znorm(x)
    err = float(np.abs(x.cpu().numpy() - gold[name + "__znorm"]).max())
    print("znorm %s: max |z - z_ref| %.2e" % (name, err))
    assert err <= 2e-6


@pytest.mark.parametrize("name", CLEAN)
@pytest.mark.parametrize("start", ["zero", "raw", "unit"])
@pytest.mark.parametrize("cal", [0, 1])
def test_extract_matches_reference(built, gpu_ctx, gold, name, start, cal):
    import torch
    T, _ = built
    n, m, k, _ = _meta(gold, name)
    C0 = {"zero": np.zeros((k, m), np.float32), "raw": gold[name + "__x"][gold[name + "__raw_rows"]],
          "unit": gold[name + "__unit"]}[start]
    c = _cuda(C0.astype(np.float32))
    counts = torch.zeros(k, dtype=torch.int32, device="cuda")
    sc = gpu_ctx.extract_shapes(_cuda(gold[name + "__xz"]), _cuda(gold[name + "__truth"].astype(np.int32)), c,
                                mode=T.MODE_COMPAT, cal_select=cal, precision=T.PREC_FP32, counts=counts)
    key = "%s__extract_%s_cal%d" % (name, start, cal)
    Cr = gold[key + "__centroids"]
    C = c.cpu().numpy()
    rel = float(np.abs(C - Cr).max() / np.abs(Cr).max())
    print("extract %s/%s/cal%d: max |c - c_ref| / max |c_ref| = %.2e" % (name, start, cal, rel))
    assert np.array_equal(counts.cpu().numpy(), gold[key + "__counts"])
    assert sc == int(gold[key + "__sum_class"][0])
    assert rel <= 1e-5


@pytest.mark.parametrize("name", CLEAN)
@pytest.mark.parametrize("init_chose,seed", [(0, 0), (1, 0), (1, 1)])
def test_loop_matches_reference(built, gpu_ctx, gold, name, init_chose, seed):
    T, _ = built
    n, m, k, cap = _meta(gold, name)
    r = gpu_ctx.kshape_run(gold[name + "__x"], k, mode=T.MODE_COMPAT, precision=T.PREC_FP32,
                           init_chose=init_chose, seed=seed, max_iter=cap)
    key = "%s__loop_i%d_s%d" % (name, init_chose, seed)
    ref_labels = gold[key + "__labels"] - 1
    iter_num, sum_class, restarted = (int(v) for v in gold[key + "__info"])
    print("loop %s init %d seed %d: labels differ %d, iterations %d (reference iter_num %d), sum_class %d/%d, "
          "restarted %d/%d" % (name, init_chose, seed, int((r["labels"] != ref_labels).sum()), r["iterations"],
                               iter_num, r["sum_class"], sum_class, r["restarted"], restarted))
    assert np.array_equal(r["labels"], ref_labels)
    assert r["sum_class"] == sum_class
    assert r["restarted"] == restarted


def test_c2_loop_matches_reference(built, gpu_ctx):
    """n = 20,000, m = 2709, k = 8 (F = 4096), init_chose=1 (mt19937 seed 1): the
    reference stops after its first assignment (<= k/2 clusters keep members), so
    its labels are those of one assignment against raw rows.  The init_chose=0
    runs are not compared: above m = 1024 the reference's norm_vec rescales a
    vector from three blocks that read it while others write it
    (shapeExtract.cuh:287-323), and two of its runs on the same input gave
    different centroids and labels (tests/test_ref_gpu_fixture.py)."""
    T, O = built
    g = np.load(GOLDEN_C2)
    x, _ = T.generate(20000, 2709, 8, noise=0.2, dirichlet=2.0, seed=1)
    if hashlib.sha256(x.tobytes()).digest() != bytes(g["x_sha256"]):
        pytest.skip("the generator gives other series on this host than where the reference ran")
    r = gpu_ctx.kshape_run(x, 8, mode=T.MODE_COMPAT, precision=T.PREC_FP32, init_chose=1, seed=1, max_iter=20)
    ref = g["labels_init1"] - 1
    info = g["info_init1"]
    print("c2 init 1: labels differ %d of 20000, sum_class %d/%d, restarted %d/%d"
          % (int((r["labels"] != ref).sum()), r["sum_class"], int(info[1]), r["restarted"], int(info[2])))
    assert np.array_equal(r["labels"], ref)
    assert r["sum_class"] == int(info[1]) and r["restarted"] == int(info[2])
