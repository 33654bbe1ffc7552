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
    "direct_local_start", "idxP2P", "idxM2L", "walk_m2l_count", "p2p_count_remote",
]


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    names = re.findall(r"^[A-Za-z_][\w \*]*?\b(\w+)\s*\([^;{]*\)\s*;", text, flags=re.M)
    return sorted(set(names))


def test_header_declares_reference_entry_points():
    names = declared_functions()
    for ref in ("fmm_construct", "fmm_prepare", "fmm_task", "fmm_ext", "fmm_deconstruct", "build_localtree",
                "p2m", "m2m", "m2l", "l2l", "l2p", "walk_m2m", "walk_l2l", "acceptance", "fmm_remote"):
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
    """The build targets sm_103a only (cuobjdump lists the ELF arch, no disassembly)."""
    cuobjdump = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "cuobjdump")
    if not os.path.exists(cuobjdump):
        return
    out = subprocess.run([cuobjdump, "--list-elf", ph.library_path()], capture_output=True, text=True).stdout
    assert "sm_103a" in out
