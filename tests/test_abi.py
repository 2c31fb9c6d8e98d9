"""CPU checks of the drop-in boundary: the C-ABI library builds for sm_103a,
loads, and exports every entry point include/lgca_gpu.h declares."""
import ctypes
import os
import re
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for hdr in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if not hdr.endswith(".h"):
            continue
        src = open(os.path.join(ROOT, "include", hdr)).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[\w\s\*]+?\b(lgca_\w+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    for must in ("lgca_create", "lgca_collide_and_propagate", "lgca_upload_state",
                 "lgca_download_state", "lgca_block_sums", "lgca_post_process",
                 "lgca_apply_body_force", "lgca_destroy"):
        assert must in names


def test_library_builds_and_exports_every_symbol():
    import lgca_gb300
    lgca_gb300.build()
    lib = ctypes.CDLL(lgca_gb300.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", lgca_gb300.LIB_PATH], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\bT (lgca_\w+)", out))
    assert set(declared_functions()) <= exported


def test_python_binding_signatures_cover_header():
    import lgca_gb300
    lgca_gb300.build()
    lib = lgca_gb300.lib()
    for n in declared_functions():
        assert getattr(lib, n).argtypes is not None, n


def test_status_strings_and_version():
    import lgca_gb300
    lgca_gb300.build()
    lib = lgca_gb300.lib()
    assert lib.lgca_abi_version() == 1
    assert lib.lgca_status_string(0) == b"ok"
    assert lib.lgca_status_string(1) == b"invalid argument"


def test_invalid_arguments_rejected_before_touching_a_device():
    import lgca_gb300
    lgca_gb300.build()
    for args in [(7, 64, 64), (1, 64, 63), (0, 0, 8), (2, -5, 8), (3, 70000, 70000)]:
        with pytest.raises(lgca_gb300.LgcaError) as e:
            lgca_gb300.GpuLattice(*args)
        assert e.value.status == 1


def test_plan_shape_rejects_invalid_shapes_before_touching_a_device():
    """lgca_plan_shape checks its arguments as lgca_create does, before it
    asks for a device; without a GPU a valid shape fails loudly."""
    import lgca_gb300
    lgca_gb300.build()
    for args in [(7, 64, 64, 10), (1, 64, 63, 10), (0, 0, 8, 10), (3, 70000, 70000, 10),
                 (0, 64, 64, -1)]:
        with pytest.raises(lgca_gb300.LgcaError) as e:
            lgca_gb300.plan_shape(*args)
        assert e.value.status == 1
    import torch
    if not torch.cuda.is_available():
        with pytest.raises(lgca_gb300.LgcaError) as e:
            lgca_gb300.plan_shape(3, 8192, 2048, 100)
        assert e.value.status != 0
