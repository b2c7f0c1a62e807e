"""The driver wrapper (ismc_gb300/dropin/drivers.py): patches for Python 3.12 /
numpy 2, the two driver-bug fixes, headless stand-ins, and execution of a
driver as __main__ with the drop-in ISMC first on sys.path.  The driver texts
here are small stand-ins written for the test that contain the constructs the
patches target; when the reference's own drivers are present they are
patched and compiled as well."""
import os
import sys

import pytest

from ismc_gb300.dropin import drivers

LOOKUP_LIKE = '''import numpy as np
import configparser
parser = configparser.SafeConfigParser()
mu_s_ = np.array([mu_s__start*mu_a_base**i for i in range(N_mu_s)])   # range of mus'
x = np.float("1.5")
diff = np.Inf
def makelookup(refl, trans):
    return 1
'''

MINIMIZATION_LIKE = '''import configparser
parser = configparser.SafeConfigParser()
if (parser.has_option('experiment','M_U_unc')):
\tT_u_exact_unc = np.array(parser.get('experiment', 'M_U_unc').split("\\n"),dtype=float)[0] # comment
else:
\tT_u_exact = None
'''


def test_patches_apply_and_compile():
    out = drivers.patch_source(LOOKUP_LIKE, "lookup.py", gpu_tables=True)
    assert "SafeConfigParser" not in out and "np.float(" not in out and "np.Inf" not in out
    assert "mu_s__start*mu_s__base**i" in out
    assert "def _reference_makelookup(" in out
    compile(out, "lookup.py", "exec")
    kept = drivers.patch_source(LOOKUP_LIKE, "lookup.py", keep_quirks=True)
    assert "mu_s__start*mu_a_base**i" in kept
    out = drivers.patch_source(MINIMIZATION_LIKE, "minimization.py")
    assert "else:\n\tT_u_exact_unc = None" in out
    compile(out, "minimization.py", "exec")


def test_patch_fails_loudly_on_other_text():
    with pytest.raises(RuntimeError):
        drivers.patch_source("print('no config parser here')\n", "minimization.py")


def test_run_driver_uses_dropin_and_stand_ins(tmp_path, monkeypatch):
    """A driver that imports ISMC the way the reference's do gets the drop-in,
    and its plotting / HDF5 calls run headless."""
    d = tmp_path / "Minimization"
    d.mkdir()
    drv = d / "minimization.py"
    drv.write_text(MINIMIZATION_LIKE.replace("if (", "import sys\nsys.path.append('../')\n"
                                             "from ISMC import ISMC as pythonISMC\nif (", 1) +
                   "import numpy as np\nRESULT = pythonISMC.__module__\n")
    monkeypatch.setattr(sys, "path", list(sys.path))
    monkeypatch.setattr(sys, "argv", list(sys.argv))
    cwd = os.getcwd()
    saved = {k: sys.modules.get(k) for k in ("ISMC",)}
    try:
        g = drivers.run_driver(str(drv), [])
    finally:
        os.chdir(cwd)
        for k, v in saved.items():
            if v is None:
                sys.modules.pop(k, None)
            else:
                sys.modules[k] = v
    assert g["RESULT"] == "ISMC"
    assert os.path.dirname(sys.modules.get("ISMC", None).__file__ if "ISMC" in sys.modules else
                           drivers.HERE + "/x") == drivers.HERE
    drivers.install_stand_ins()
    import matplotlib.pyplot as plt        # real or stand-in
    fig, ax = plt.subplots()
    import hdf5storage
    if hasattr(hdf5storage, "__getattr__"):
        hdf5storage.write({"a": [1, 2]}, str(tmp_path), "t.h5", matlab_compatible=True)
        assert (tmp_path / "t.npz").exists()


def _reference_dir():
    from oracle import build_ref
    return build_ref.reference_dir()


@pytest.mark.skipif(_reference_dir() is None, reason="reference drivers not present")
def test_reference_drivers_patch_and_compile():
    REF = _reference_dir()
    for name, sub in (("lookup.py", "Lookup"), ("minimization.py", "Minimization")):
        p = os.path.join(REF, sub, name)
        with open(p) as f:
            src = f.read()
        out = drivers.patch_source(src, name, gpu_tables=(name == "lookup.py"))
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore", SyntaxWarning)
            compile(out, p, "exec")
