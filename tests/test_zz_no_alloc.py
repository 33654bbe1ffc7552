"""photons_direct_sum_noalloc: the FP64 direct sum for callers that cannot
allocate device memory while they run (a simulation that has given all of
HBM to its particles, PM mesh and force-pass pools, or that must not stall
its other streams with the device-wide synchronisation of cudaMalloc and
cudaFree).  Inputs and outputs are device buffers the caller already owns;
the scratch is a fixed array inside the library.

Called through the C ABI and compared with photons_direct_sum, the
allocating entry point, on two calls in a row with different sizes, so the
second call also shows that the shared scratch is cleared between calls.
This file sorts last so that a run stopping at the first failure has run
every other test before it."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-10  # the FP64 direct-sum parity bound of the other GPU tests


def rel_err(a, b, p, n):
    """|a-b|/|b| per target, floored at 1e-4 of one mean-spacing pair force
    m/D^2 (D = L/n^(1/3)) where the net force cancels."""
    nb = np.linalg.norm(b, axis=1)
    spacing = p["boxsize"] / np.cbrt(n)
    floor = 1e-4 * p["mass"] / spacing ** 2
    return np.linalg.norm(a - b, axis=1) / np.maximum(nb, floor)


@pytest.fixture(scope="module")
def noalloc(ph):
    lib = C.CDLL(ph.library_path())
    f = lib.photons_direct_sum_noalloc
    f.restype = C.c_int
    f.argtypes = [C.POINTER(ph.Params), C.c_int, C.c_void_p, C.c_int, C.c_void_p, C.c_double, C.c_void_p,
                  C.c_void_p]
    lib.photons_gpu_error.restype = C.c_char_p
    return lib


def _call(lib, ph, p, dpos, dtargets, dacc, rmax, n=None, nt=None):
    prm = ph.make_params(p)
    n = dpos.shape[0] if n is None else n
    nt = dtargets.shape[0] if nt is None else nt
    rc = lib.photons_direct_sum_noalloc(C.byref(prm), n, dpos.data_ptr(), nt, dtargets.data_ptr(), float(rmax),
                                        dacc.data_ptr(), None)
    return rc, lib.photons_gpu_error().decode(errors="replace")


def test_noalloc_matches_direct_sum_two_calls(ph, ics, noalloc):
    torch = pytest.importorskip("torch")
    # 8^3 cells of side >= rmax, then 4^3 cells and fewer sources
    cases = [ics.make("nfw128", nside=48), ics.make("nfw128", nside=24)]
    rng = np.random.default_rng(11)
    for k, (pos, p) in enumerate(cases):
        targets = rng.choice(pos.shape[0], 700 - 200 * k, replace=False).astype(np.int32)
        rmax = p["rcut"]
        want = ph.direct_sum(pos, p, targets, rmax)
        dpos = torch.from_numpy(np.ascontiguousarray(pos, np.float64)).cuda()
        dtargets = torch.from_numpy(targets).cuda()
        dacc = torch.full((targets.size, 3), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc, msg = _call(noalloc, ph, p, dpos, dtargets, dacc, rmax)
        assert rc == 0, msg
        got = dacc.cpu().numpy()
        assert np.isfinite(got).all()
        assert rel_err(got, want, p, pos.shape[0]).max() <= TOL, f"call {k + 1}"


def test_noalloc_allocates_nothing_after_warm_up(ph, ics, noalloc):
    """After the warm-up call (nt = 0: set-up only) a call leaves the
    device's free memory unchanged, i.e. it allocated nothing."""
    torch = pytest.importorskip("torch")
    pos, p = ics.make("nfw128", nside=32)
    dpos = torch.from_numpy(np.ascontiguousarray(pos, np.float64)).cuda()
    dtargets = torch.arange(0, pos.shape[0], 97, dtype=torch.int32, device="cuda")
    dacc = torch.empty((dtargets.shape[0], 3), dtype=torch.float64, device="cuda")
    rc, msg = _call(noalloc, ph, p, dpos, dtargets, dacc, p["rcut"], nt=0)
    assert rc == 0, msg
    rc, msg = _call(noalloc, ph, p, dpos, dtargets, dacc, p["rcut"])  # first real call after the set-up
    assert rc == 0, msg
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    stats0 = torch.cuda.memory_stats().get("allocation.all.allocated", 0)
    for _ in range(3):
        rc, msg = _call(noalloc, ph, p, dpos, dtargets, dacc, p["rcut"])
        assert rc == 0, msg
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert torch.cuda.memory_stats().get("allocation.all.allocated", 0) == stats0


def test_noalloc_rejects_bad_input(ph, ics, noalloc):
    torch = pytest.importorskip("torch")
    pos, p = ics.make("grid32", nside=8)
    dpos = torch.from_numpy(np.ascontiguousarray(pos, np.float64)).cuda()
    dtargets = torch.arange(4, dtype=torch.int32, device="cuda")
    dacc = torch.empty((4, 3), dtype=torch.float64, device="cuda")
    # sizes beyond the fixed scratch are refused on the host, before any launch
    rc, msg = _call(noalloc, ph, p, dpos, dtargets, dacc, p["rcut"], n=(1 << 18) + 1)
    assert rc == 1 and "maximum" in msg
    rc, msg = _call(noalloc, ph, p, dpos, dtargets, dacc, p["rcut"], nt=(1 << 16) + 1)
    assert rc == 1 and "maximum" in msg
    # host buffers are refused
    hpos = np.ascontiguousarray(pos, np.float64)
    prm = ph.make_params(p)
    rc = noalloc.photons_direct_sum_noalloc(C.byref(prm), pos.shape[0], hpos.ctypes.data, 4, dtargets.data_ptr(),
                                            float(p["rcut"]), dacc.data_ptr(), None)
    assert rc == 1 and "device pointers" in noalloc.photons_gpu_error().decode()
    # an out-of-range target is caught by the kernel's own bounds check
    bad = torch.tensor([0, 1, pos.shape[0], 3], dtype=torch.int32, device="cuda")
    rc, msg = _call(noalloc, ph, p, dpos, bad, dacc, p["rcut"])
    assert rc == 1 and "out of range" in msg
    # and the next call is clean again
    rc, msg = _call(noalloc, ph, p, dpos, dtargets, dacc, p["rcut"])
    assert rc == 0, msg
