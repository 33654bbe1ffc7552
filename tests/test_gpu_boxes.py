"""Many independent periodic boxes in one pass (photons_force_pass_boxes):
one tree root per box, one launch per operator for all boxes.  Each box is
its own periodic domain with its own side, rs, rcut, softening and mass, so
the batched pass must reproduce separate passes over the boxes exactly, in
FP64 and in FP32 split precision."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SUMMED = ("idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "nleaf", "nnode", "pairs_local", "pairs_image")


def _boxes(ics, nbox=7, maxleaf=12):
    out = []
    for pos, p in ics.plummer_boxes(nbox=nbox, seed=4, nmin=12 ** 3, nmax=22 ** 3):
        p = dict(p, maxleaf=maxleaf, theta=0.5)
        out.append((pos, p))
    return out


@pytest.mark.parametrize("precision", ["FP64", "FP32_SPLIT"])
def test_boxes_match_separate_passes(ph, ics, precision):
    prec = getattr(ph, precision)
    boxes = _boxes(ics)
    assert len({p["boxsize"] for _, p in boxes}) == len(boxes)  # genuinely different boxes
    fp = ph.ForcePass(0)
    got = fp.run_boxes(boxes, precision=prec)
    cb = fp.counters()
    sums = {k: 0 for k in SUMMED}
    one = ph.ForcePass(0)
    for (pos, p), g in zip(boxes, got):
        want = one.run(pos, p, precision=prec)
        assert np.array_equal(g, want)
        c = one.counters()
        for k in SUMMED:
            sums[k] += c[k]
    for k in SUMMED:
        assert cb[k] == sums[k], k


@pytest.mark.parametrize("maxleaf", [48, 64])
def test_boxes_mutual_pairs_match_separate_passes(ph, ics, maxleaf):
    """From leaf 48 the FP32 pass evaluates each symmetric leaf pair once
    (reactions through per-pair slots).  Pairing never crosses boxes and
    keeps each box's leaf order, so the batched pass still equals the
    separate passes bit for bit."""
    boxes = [(pos, dict(p, maxleaf=maxleaf, theta=0.5))
             for pos, p in ics.plummer_boxes(nbox=4, seed=6, nmin=24 ** 3, nmax=32 ** 3)]
    got = ph.ForcePass(0).run_boxes(boxes, precision=ph.FP32_SPLIT)
    one = ph.ForcePass(0)
    for (pos, p), g in zip(boxes, got):
        assert np.array_equal(g, one.run(pos, p, precision=ph.FP32_SPLIT))


def test_boxes_graph_and_stage_paths_agree(ph, ics, monkeypatch):
    boxes = _boxes(ics, nbox=4)
    a = ph.ForcePass(0).run_boxes(boxes, precision=ph.FP32_SPLIT)
    monkeypatch.setenv("PHOTONS_GRAPH", "0")
    b = ph.ForcePass(0).run_boxes(boxes, precision=ph.FP32_SPLIT)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_boxes_reuse_one_graph_for_new_box_constants(ph, ics):
    """The box table is read on the device: the same counts with other box
    sides and masses reuse the captured pass and still give the right forces."""
    boxes = _boxes(ics, nbox=3)
    fp = ph.ForcePass(0)
    fp.run_boxes(boxes, precision=ph.FP64)
    scaled = [(pos * 1.5, dict(p, boxsize=p["boxsize"] * 1.5, mass=p["mass"] * 2.0, rs=p["rs"] * 1.5,
                               rcut=p["rcut"] * 1.5, eps=p["eps"] * 1.5)) for pos, p in boxes]
    got = fp.run_boxes(scaled, precision=ph.FP64)
    one = ph.ForcePass(0)
    for (pos, p), g in zip(scaled, got):
        assert np.array_equal(g, one.run(pos, p, precision=ph.FP64))


def test_boxes_reject_mixed_opening_angles(ph, ics):
    boxes = _boxes(ics, nbox=2)
    pos0, p0 = boxes[0]
    pos1, p1 = boxes[1]
    fp = ph.ForcePass(0)
    prm = (ph.Params * 2)(ph.make_params(p0, ph.FP64), ph.make_params(dict(p1, theta=0.7), ph.FP64))
    counts = np.array([pos0.shape[0], pos1.shape[0]], np.int32)
    pos = np.ascontiguousarray(np.concatenate([pos0, pos1]))
    acc = np.empty_like(pos)
    import ctypes as C
    rc = fp.lib.photons_force_pass_boxes(fp.h, 2, prm, counts.ctypes.data_as(C.POINTER(C.c_int)), pos.ctypes.data,
                                         acc.ctypes.data)
    assert rc == 1
    assert "must match" in fp.lib.photons_gpu_error().decode()
