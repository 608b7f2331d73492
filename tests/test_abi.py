"""The C-ABI library: builds, loads and exports every entry point the header
declares; the ctypes structs match the C layout; host-only entry points
(constants, coefficient table) agree bit for bit with the oracle; without a
GPU, fs_create fails cleanly with FS_ERR_NO_DEVICE.  No device compute here."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from fluidsim_gb300 import abi, api, config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "fluidsim_gpu.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fs_[a-z_0-9]+)\s*\(", txt)))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("fs_create", "fs_destroy", "fs_ptcl_step", "fs_lapl_solve", "fs_accept",
              "fs_reject", "fs_upload_state", "fs_download_state", "fs_run"):
        assert n in names


def test_library_exports_every_symbol(built):
    lib = C.CDLL(api.lib_path())
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", api.lib_path()], capture_output=True, text=True)
    for n in declared_functions():
        assert re.search(r"\bT %s\b" % n, out.stdout), n


def test_struct_layout_matches_c(tmp_path):
    src = tmp_path / "sizes.c"
    src.write_text(
        '#include <stdio.h>\n#include <stddef.h>\n#include "fluidsim_gpu.h"\n'
        'int main(void){printf("%zu %zu %zu %zu %zu %zu\\n", sizeof(fs_config), sizeof(fs_mesh),'
        ' sizeof(fs_constants), sizeof(fs_stats), offsetof(fs_config, table_emin_ev),'
        ' offsetof(fs_stats, steps)); return 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    vals = [int(v) for v in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert vals == [C.sizeof(abi.FsConfig), C.sizeof(abi.FsMesh), C.sizeof(abi.FsConstants),
                    C.sizeof(abi.FsStats), abi.FsConfig.table_emin_ev.offset, abi.FsStats.steps.offset]


def test_abi_version(built):
    assert api.load_library().fs_abi_version() == abi.FS_ABI_VERSION


@pytest.mark.parametrize("p,gam", [(1.0, 0.07), (10.0, 0.1), (0.5, 0.03)])
def test_constants_and_table_match_oracle(built, p, gam):
    from oracle import oracle
    cfg = config.glow(16, p_torr=p, gam=gam)
    kp = api.constants(cfg)
    ko = api.constants(cfg, oracle.load(), "or_")
    assert kp == ko
    tp = api.coefficient_table(cfg)
    to = api.coefficient_table(cfg, oracle.load(), "or_")
    assert np.array_equal(tp, to)
    assert np.all(np.isfinite(tp)) and np.all(tp[[0, 1, 2, 4, 5]] > 0)


def test_create_without_device_fails_cleanly(built):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(api.FluidsimError) as ei:
        api.Discharge(config.glow(8))
    assert ei.value.code == abi.FS_ERR_NO_DEVICE


def test_invalid_config_rejected_before_device(built):
    good = config.glow(8)
    cfg = good.replace(nx=2)
    with pytest.raises(api.FluidsimError) as ei:
        api.Discharge(cfg, good.mesh())
    assert ei.value.code == abi.FS_ERR_UNSUPPORTED
    for bad, code in ((dict(rf=7), abi.FS_ERR_UNSUPPORTED), (dict(rf=1, res=0.0), abi.FS_ERR_INVALID),
                      (dict(precision=5), abi.FS_ERR_INVALID),
                      (dict(coef_mode=abi.FS_COEF_FITS, precision=abi.FS_PREC_MIXED), abi.FS_ERR_UNSUPPORTED)):
        cfg = config.glow(8).replace(**bad)
        with pytest.raises(api.FluidsimError) as ei:
            api.Discharge(cfg)
        assert ei.value.code == code, bad


def test_null_context_rejected(built):
    """The configuration and driver entry points refuse a null context (or
    context array) with FS_ERR_INVALID before touching a device."""
    lib = api.load_library()
    assert lib.fs_set_line_smoother(None, 0) == abi.FS_ERR_INVALID
    assert lib.fs_line_smoother(None) == -1
    assert lib.fs_set_stage_tile(None, 32, 8) == abi.FS_ERR_INVALID
    st = (abi.FsStats * 1)()
    rc = (C.c_int32 * 1)()
    assert lib.fs_batch_run(None, 1, 1, 0.0, 1, st, rc) == abi.FS_ERR_INVALID
    assert lib.fs_batch_run_fused(None, 1, 1, 0.0, 1, st, rc) == abi.FS_ERR_INVALID
    arr = (C.c_void_p * 1)(None)
    assert lib.fs_batch_run_fused(arr, 1, 1, 0.0, 1, st, rc) == abi.FS_ERR_INVALID
