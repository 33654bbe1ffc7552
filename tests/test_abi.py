"""The C-ABI library loads and exports every function declared in
include/photons_fmm.h and the reference's globals.  No GPU calls."""
import ctypes
import os
import re
import subprocess

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "photons_fmm.h")

REFERENCE_GLOBALS = [
    "part", "btree", "leaf", "toptree", "open_angle", "first_node", "last_node", "first_leaf", "last_leaf",
    "MAXLEAF", "PROC_RANK", "PROC_SIZE", "BOXSIZE", "NPART", "NLEAF", "NNODE", "NPART_TOTAL", "MASSPART",
    "SoftenScale", "cutoffRadius", "splitRadius", "first_domain", "last_domain", "this_domain", "mostleft",
    "direct_local_start", "idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote", "NSIDE",
]


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for ref in ("fmm_construct", "fmm_prepare", "fmm_task", "fmm_ext", "fmm_deconstruct", "build_localtree",
                "p2m", "m2m", "m2l", "l2l", "l2p", "walk_m2m", "walk_l2l", "acceptance", "fmm_remote",
                "partmesh_thread", "partmesh", "pm_thread", "get_local_size_", "p2p_kernel", "p2p_kernel_inleaf",
                "p2p_kernel_rinvsqrt"):
        assert ref in names


def test_library_exports_every_declared_symbol(ph):
    lib = ctypes.CDLL(ph.library_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_library_exports_reference_globals(ph):
    out = subprocess.run(["nm", "-D", "--defined-only", ph.library_path()], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if line.strip()}
    missing = [g for g in REFERENCE_GLOBALS if g not in exported]
    assert not missing, missing


def test_library_is_sm103a(ph):
    """The build compiles every source for sm_103a alone (one -gencode, no PTX
    for other architectures) and the library it links is present."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("pkg_build", os.path.join(os.path.dirname(ph.library_path()),
                                                                            os.pardir, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    assert b.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]
    assert not any("gencode" in f or "arch=" in f for f in b.FLAGS)
    assert os.path.exists(ph.library_path())
