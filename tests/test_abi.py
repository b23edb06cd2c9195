"""The C-ABI library loads without a GPU and exports every entry point include/atsat_dyn.h declares;
the ctypes structs match the header's layout."""
import ctypes as C
import os
import re

import pytest

from atsat_gb300 import abi, fields as F

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "atsat_dyn.h")


def declared():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(atsat_dyn_\w+)\s*\(", txt)))


@pytest.fixture(scope="module")
def lib():
    from atsat_gb300 import build
    build.build()
    from atsat_gb300 import dyn
    return dyn.lib()


def test_library_exports_every_declared_symbol(lib):
    names = declared()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_field_ids_match_header():
    txt = open(HEADER).read()
    for name, value in [("ATSAT_F_P_DYN", F.P_DYN), ("ATSAT_F_NUE", F.NUE), ("ATSAT_F_RHS_BASE", F.RHS_BASE),
                        ("ATSAT_F_AUX_U", F.AUX_U), ("ATSAT_F_P_DYNN", F.P_DYNN), ("ATSAT_NFIELDS", F.NFIELDS)]:
        m = re.search(name + r"\s*=\s*(\d+)", txt)
        assert m and int(m.group(1)) == value, name


def test_params_struct_matches_defaults(lib):
    p = abi.Params()
    assert lib.atsat_dyn_params_default(C.byref(p)) == 0
    want = abi.default_params()
    for n, _ in F.PARAM_DOUBLES:
        assert getattr(p, n) == want[n], n
    for n, _ in F.PARAM_INTS:
        assert getattr(p, n) == want[n], n


def test_params_from_env_resolves_like_the_reference(lib, monkeypatch):
    from atsat_gb300 import dyn
    for k in list(os.environ):
        if k.startswith("ATSAT_"):
            monkeypatch.delenv(k)
    p = dyn.params_from_env()
    assert p["press_incr"] == 1 and p["nd_cor"] == 1 and p["cell_hold"] == 1 and p["turb_active"] == 1
    monkeypatch.setenv("ATSAT_GEO_BALANCE", "0")
    p = dyn.params_from_env()
    assert p["press_incr"] == 0 and p["nd_cor"] == 0 and p["cell_hold"] == 0
    monkeypatch.setenv("ATSAT_NONDIM", "1")
    p = dyn.params_from_env()
    assert p["nd_cor"] == 1 and p["nd_cent"] == 1 and p["nd_buoy"] == 1
    monkeypatch.setenv("ATSAT_METRIC_SPLIT", "0")
    p = dyn.params_from_env()
    assert p["metric_split"] == 0 and p["coriolis_split"] == 0
    monkeypatch.setenv("ATSAT_TURB_MODEL", "none")
    assert dyn.params_from_env()["turb_active"] == 0
    monkeypatch.setenv("ATSAT_PRESS_SWEEPS", "-3")
    assert dyn.params_from_env()["press_sweeps"] == 1
    monkeypatch.setenv("ATSAT_BC_SEAM_DAMP", "2")
    with pytest.raises(dyn.DycoreError):
        dyn.params_from_env()


def test_create_without_gpu_fails_loudly(lib):
    """No CPU fallback: without a usable GPU, create returns a CUDA status, never a silent handle."""
    from atsat_gb300 import dyn, synth
    import shutil
    import subprocess
    smi = shutil.which("nvidia-smi")
    if smi and subprocess.run([smi], capture_output=True).returncode == 0:
        pytest.skip("a GPU is present")
    with pytest.raises(dyn.DycoreError) as e:
        dyn.Dycore(synth.make_grid(9, 13, 17), abi.default_params())
    assert e.value.status == abi.E_CUDA


def test_unsupported_knobs_are_rejected(lib):
    from atsat_gb300 import dyn, synth
    with pytest.raises(dyn.DycoreError) as e:
        dyn.Dycore(synth.make_grid(9, 13, 17), abi.default_params(chrom=1))
    assert e.value.status == abi.E_UNSUPPORTED
    # the split Coriolis form without the metric split: the reference forces it off, the device refuses it
    with pytest.raises(dyn.DycoreError) as e:
        dyn.Dycore(synth.make_grid(9, 13, 17), abi.default_params(metric_split=0, coriolis_split=1))
    assert e.value.status == abi.E_UNSUPPORTED


def test_autotune_cache_read_and_write(lib, tmp_path):
    """The autotune cache file: a key is absent until written, the latest write of a key wins, other keys
    (grid, source knobs, GPU model) are kept apart, and GPU names with blanks are stored as one token."""
    path = str(tmp_path / "sub" / "tune.txt").encode()
    v, lv, ms = C.c_int32(-1), C.c_int32(0), C.c_double(0.0)

    def get(im, jm, km, knobs, gpu):
        return lib.atsat_dyn_tune_cache_get(path, im, jm, km, knobs, gpu, C.byref(v), C.byref(lv), C.byref(ms))

    assert get(41, 181, 361, 5, b"NVIDIA GB300") == abi.E_INVALID
    assert lib.atsat_dyn_tune_cache_put(path, 41, 181, 361, 5, b"NVIDIA GB300", 7, 39, 0.25) == abi.OK
    assert lib.atsat_dyn_tune_cache_put(path, 21, 91, 181, 5, b"NVIDIA GB300", 6, 0, 0.05) == abi.E_INVALID
    assert lib.atsat_dyn_tune_cache_put(path, 21, 91, 181, 5, b"NVIDIA GB300", 7, 4, 0.05) == abi.OK
    assert get(41, 181, 361, 5, b"NVIDIA GB300") == abi.OK and (v.value, lv.value) == (7, 39)
    assert abs(ms.value - 0.25) < 1e-9
    assert get(41, 181, 361, 1, b"NVIDIA GB300") == abi.E_INVALID
    assert get(41, 181, 361, 5, b"NVIDIA B200") == abi.E_INVALID
    assert lib.atsat_dyn_tune_cache_put(path, 41, 181, 361, 5, b"NVIDIA GB300", 6, 20, 0.30) == abi.OK
    assert get(41, 181, 361, 5, b"NVIDIA GB300") == abi.OK and (v.value, lv.value) == (6, 20)
    assert get(21, 91, 181, 5, b"NVIDIA GB300") == abi.OK and (v.value, lv.value) == (7, 4)
    lines = open(path.decode()).read().splitlines()
    assert len(lines) == 2 and all("NVIDIA_GB300" in ln for ln in lines)
