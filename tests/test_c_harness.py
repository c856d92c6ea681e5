"""The C-ABI compiles and links from plain C (the way a Fortran shim or
another language binds it) and its host-only paths work without a GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIBDIR = os.path.join(ROOT, "standalone_mgbf_loc_gb300", "_lib")

NML = """&PARAMETERS_MGBETA
  mg_ampl01=2.0, mg_ampl02=5.28125, mg_ampl03=1.0,
  mg_weig1=1.,mg_weig2=0.5,mg_weig3=0.25,mg_weig4=0.125,mg_weig5=0.0625,
  hx=6,hy=6,hz=3,p=2, mgbf_line=.false., mgbf_proc=1, n_ens=1,
  lm_a=16, lm=16, km2=0, km3=1, l_filt_g1=.true., l_vertical_filter=.true.,
  lquart=.false., lhelm=.false., gm_max=3, nm0=0, mm0=0,
  nxPE=4, nyPE=4, im_filt=16, jm_filt=16,
/
"""


def build_harness(lib, tmp_path):
    if not shutil.which("gcc"):
        pytest.skip("gcc missing")
    exe = tmp_path / "abi_harness"
    subprocess.run(["gcc", "-std=c99", "-O1", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "c", "abi_harness.c"), "-L", LIBDIR, "-lmgbf",
                    "-Wl,-rpath," + LIBDIR, "-lm", "-o", str(exe)], check=True)
    (tmp_path / "mgbeta.nml").write_text(NML)
    return exe


def test_c_harness_host_only(lib, tmp_path):
    exe = build_harness(lib, tmp_path)
    r = subprocess.run([str(exe), "host", str(tmp_path / "mgbeta.nml")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "im=64 jm=64 km_all=16 gm=3 reach_h=6 reach_z=3" in r.stdout
    assert r.stdout.strip().endswith("ok")


@pytest.mark.gpu
def test_c_harness_gpu_impulse(lib, tmp_path):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    import numpy as np
    from oracle import oracle as O
    from standalone_mgbf_loc_gb300.mgbf import MGBFConfig
    from tests.helpers import oracle_cfg, rel_l2
    exe = build_harness(lib, tmp_path)
    out = tmp_path / "vall.bin"
    r = subprocess.run([str(exe), "gpu", str(tmp_path / "mgbeta.nml"), str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "impulse response" in r.stdout
    # the same impulse (grid centre, level 1) through the oracle's
    # filtering_procedure(1) on VALL with its halo
    cfg = oracle_cfg(MGBFConfig.from_namelist(str(tmp_path / "mgbeta.nml")), 1)
    v = np.zeros((cfg.J + 2 * cfg.hy, cfg.I + 2 * cfg.hx, cfg.nk))
    v[cfg.J // 2 + cfg.hy, cfg.I // 2 + cfg.hx, 0] = 1.0
    O.filtering_procedure(cfg, v)
    got = np.fromfile(out, dtype=np.float64).reshape(v.shape)
    assert rel_l2(got, v) < 1e-12
