"""The C-ABI library on a CPU-only machine: it loads, exports every function
include/*.h declares, refuses to run without a device, and its host-side tree
and interaction lists equal the oracle's exactly."""
import ctypes as C
import dataclasses
import glob
import os
import re

import numpy as np
import pytest

import hsr
import synth
from hsr_testutil import golden_names, load_golden, same_lists

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"^\s*(?:hsr_status|const char \*|void)\s*\**\s*(hsr_\w+)\s*\(",
                                text, flags=re.M))
    return sorted(names)


def test_header_declares_functions():
    assert len(header_functions()) >= 10


def test_every_entry_point_names_what_it_replaces():
    """Each declaration's comment cites the reference (file:line) or says it
    has no counterpart there."""
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    missing = []
    for h in sorted(glob.glob(os.path.join(root, "include", "hacc_*.h"))):
        src = open(h).read()
        for m in re.finditer(r"/\*((?:(?!\*/).)*)\*/\s*hsr_status\s+(hsr_\w+)\s*\(", src, re.S):
            doc = re.sub(r"\s*\n\s*\*?\s*", "", m.group(1))
            if not re.search(r"\.(cxx|c|h|cpp|hpp):\d", doc) and "counterpart" not in doc:
                missing.append(m.group(2))
    assert not missing, missing


def test_library_binds_every_symbol_at_load(hsr_lib):
    """The library loads with every symbol bound at once (no symbol of its
    own left undefined by a definition in the wrong namespace)."""
    import ctypes
    import os
    ctypes.CDLL(hsr.LIB_PATH, mode=os.RTLD_NOW | os.RTLD_LOCAL)


@pytest.mark.parametrize("name", header_functions())
def test_library_exports(hsr_lib, name):
    assert hasattr(hsr_lib, name), f"{name} declared in include/ but not exported"


def test_python_binding_lists_every_export(hsr_lib):
    assert set(header_functions()) == set(hsr.EXPORTS)


def test_version(hsr_lib):
    assert b"sm_103a" in hsr_lib.hsr_version()


def _has_gpu():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_gpu(), reason="a CUDA device is present")
def test_create_without_device_fails_loudly(hsr_lib):
    h = C.c_void_p()
    assert hsr_lib.hsr_create(C.byref(h), 0) == 6  # HSR_ERR_NO_DEVICE
    with pytest.raises(hsr.HsrError):
        hsr.Context(0)


@pytest.mark.parametrize("name", golden_names())
def test_host_tree_permutation_matches_golden(hsr_lib, name):
    p, kp, out = load_golden(name)
    L = hsr.HostLists(p, kp)
    for k in ("x", "y", "z", "mass", "phi", "id", "mask"):
        assert np.array_equal(getattr(p, k).view(np.uint8), out[k].view(np.uint8)), f"{name}: {k}"
    assert L.nleaves >= 1 or p.n == 0


@pytest.mark.parametrize("case", ["zel16_nd32", "zel16_nd16_quad", "zel16_oa05_nd8", "random_nd1",
                                  "long_chains", "zel16_nd32_rco", "zel16_nd16_quad_rco",
                                  "clustered16_oa05_nd8_rco"])
def test_host_lists_equal_oracle_lists(hsr_lib, oracle_lib, case):
    """The host build (RCB, and the RCO octree where the case says so)
    against the oracle: permutation, list entries and pair counts exact."""
    if case == "long_chains":
        p = synth.sorted_line(20000)
        kp = synth.kick_params(p, nd=32)
        kp.min_force, kp.max_force = (1.0, 0.0, 0.0), (39.0, 0.5, 0.5)
    elif case.startswith("zel16") or case.startswith("clustered16"):
        p = (synth.zeldovich_box(16, z=10.0, seed=4) if case.startswith("zel16")
             else synth.clustered_box(16, nhalo=20, seed=15))
        nd = int(case.split("nd")[-1].split("_")[0])
        kp = synth.kick_params(p, nd=nd, tdpts=12 if "quad" in case else 1,
                               open_angle=0.5 if "oa05" in case else 0.1)
    else:
        p = synth.random_box(600, 8.0, 3)
        kp = synth.kick_params(p, nd=1)
        kp.min_force, kp.max_force = (0.5,) * 3, (7.5,) * 3
    if case.endswith("_rco"):
        kp = dataclasses.replace(kp, tree=hsr.TREE_RCO)
    q = p.copy()
    L = hsr.HostLists(p, kp)
    r = oracle_lib.rcb_run(q, kp, keep_lists=True, do_kick=False, nthreads=2)
    for k in ("x", "y", "z", "mass", "phi", "id", "mask", "vx"):
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
    off, cnt, ptr, e = L.get()
    ooff, ocnt, optr = r.leaves()
    assert L.stats["pairs"] == r.stats["pairs"]
    assert L.stats["list_entries"] == r.stats["list_entries"]
    assert same_lists(off, cnt, ptr, e, ooff, ocnt, optr, r.entries())
    assert L.stats["nodes"] == r.stats["nodes"]


@pytest.mark.parametrize("tdpts,tree", [(1, 0), (12, 0), (1, 1), (12, 1)])
def test_host_lists_with_signed_zero_coordinates(hsr_lib, oracle_lib, tdpts, tree):
    """A third of the coordinates on the planes x, y, z = 0 with both signs
    of zero (the node bounds tie at zeros of either sign): the host build's
    permutation and lists equal the oracle's bit for bit."""
    p = synth.random_box(3000, 8.0, 2)
    rng = np.random.default_rng(102)
    for a in (p.x, p.y, p.z):
        sel = rng.random(p.n) < 0.3
        a[sel] = np.where(rng.random(int(sel.sum())) < 0.5, np.float32(0.0), np.float32(-0.0))
    kp = synth.kick_params(p, nd=8, tdpts=tdpts, open_angle=0.5)
    kp.min_force, kp.max_force = (-1.0,) * 3, (7.0,) * 3
    kp = dataclasses.replace(kp, tree=tree)
    q = p.copy()
    L = hsr.HostLists(p, kp)
    r = oracle_lib.rcb_run(q, kp, keep_lists=True, do_kick=False, nthreads=2)
    for k in ("x", "y", "z", "mass", "phi", "id", "mask"):
        assert np.array_equal(getattr(p, k).view(np.uint8), getattr(q, k).view(np.uint8)), k
    off, cnt, ptr, e = L.get()
    ooff, ocnt, optr = r.leaves()
    assert L.stats["pairs"] == r.stats["pairs"]
    assert same_lists(off, cnt, ptr, e, ooff, ocnt, optr, r.entries())


def test_host_lists_index_points_at_entries(hsr_lib):
    p = synth.zeldovich_box(8, seed=2)
    kp = synth.kick_params(p, nd=16)
    L = hsr.HostLists(p, kp)
    off, cnt, ptr, e = L.get()
    idx = L.index()
    real = idx < p.n
    assert np.array_equal(e[0][real], p.x[idx[real]])
    assert np.array_equal(e[3][real], p.mass[idx[real]])


@pytest.mark.parametrize("bad", ["tdpts", "nd", "n", "null"])
def test_bad_arguments_rejected(hsr_lib, bad):
    p = synth.random_box(10, 4.0, 1)
    kp = synth.kick_params(p, nd=4)
    P = hsr.make_params(kp)
    args = hsr._particle_args(p)
    n = p.n
    if bad == "tdpts":
        P.tdpts = 3
    elif bad == "nd":
        P.nd = 0
    elif bad == "n":
        n = -1
    else:
        args[3] = C.cast(None, C.POINTER(C.c_float))
    h = C.c_void_p()
    assert hsr_lib.hsr_build_lists(C.byref(P), n, *args, C.byref(h)) == 1
    assert not h.value


@pytest.mark.parametrize("case", ["empty", "one", "coincident", "nd1", "big_leaf"])
def test_host_work_items_cover_every_leaf_particle(hsr_lib, case):
    """Batched work items: one per group of <= 32 particles of each processed
    leaf (times list chunks); empty leaves get none."""
    if case == "empty":
        p = synth.random_box(0, 4.0, 1)
    elif case == "one":
        p = synth.random_box(1, 4.0, 1)
    elif case == "coincident":
        p = synth.random_box(300, 4.0, 1)
        p.x[:200] = 2.0
        p.y[:200] = 2.0
        p.z[:200] = 2.0
    elif case == "nd1":
        p = synth.random_box(400, 6.0, 2)
    else:
        p = synth.random_box(3000, 6.0, 2)
    kp = synth.kick_params(p, nd={"nd1": 1, "big_leaf": 5000}.get(case, 16), fcoeff=1.0)
    kp.min_force, kp.max_force = (-1.0,) * 3, (9.0,) * 3
    L = hsr.HostLists(p, kp)
    off, cnt, ptr, e = L.get()
    lens = np.diff(ptr)
    chunks = np.maximum(1, (lens + 8191) // 8192)
    assert L.stats["work_items"] == int((((cnt + 31) // 32) * chunks).sum())
