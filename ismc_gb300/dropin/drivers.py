"""Run the reference's unmodified driver scripts (Lookup/lookup.py,
Minimization/minimization.py) on this engine under Python 3.12 / numpy 2.

    python -m ismc_gb300.dropin.drivers path/to/Lookup/lookup.py --Python example.ini
    python -m ismc_gb300.dropin.drivers path/to/Minimization/minimization.py --CUDA \\
        --CUDAsource ismc_gb300/bin/minimize.o --GPU 0 example.ini

The driver file is read, patched in memory (never on disk) and executed as
`__main__` with its own directory as the working directory:

  * `from ISMC import ISMC` resolves to this package's drop-in
    (ismc_gb300/dropin/ISMC.py, the GPU propagator), which is put on sys.path
    ahead of the driver's own `sys.path.append("../")`;
  * removed APIs are replaced: configparser.SafeConfigParser -> ConfigParser
    (lookup.py:45, minimization.py:38), np.float -> float (lookup.py:197,203),
    np.Inf -> np.inf (lookup.py:468,474);
  * two driver bugs are fixed unless keep_quirks is set: minimization.py:80-83
    sets T_u_exact = None when M_U_unc is absent (meant T_u_exact_unc), and
    lookup.py:126 builds the mu_s' axis with mu_a_base instead of mu_s__base;
  * modules the image lacks get headless stand-ins: matplotlib (plots are not
    drawn), h5py, and hdf5storage (hdf5storage.write saves the same keys to
    an .npz file beside the requested .h5 name);
  * with gpu_tables, lookup.py's makelookup (cubic griddata and a Python
    Monte Carlo uncertainty loop) is replaced by ismc_gb300.lookup.make_lookup
    (the same Clough-Tocher interpolation and uncertainty map on the GPU).

Every patch asserts that the text it replaces is present, so a driver of a
different version fails loudly instead of running half-patched.
"""
import argparse
import importlib
import os
import re
import sys
import types
import warnings

HERE = os.path.dirname(os.path.abspath(__file__))


class _Noop:
    """Accepts any attribute access, call, item access or `a, b = x` unpacking."""

    def __getattr__(self, name):
        return _Noop()

    def __call__(self, *a, **k):
        return _Noop()

    def __getitem__(self, k):
        return _Noop()

    def __iter__(self):
        return iter((_Noop(), _Noop()))


def _stub_module(name, **attrs):
    m = types.ModuleType(name)
    m.__getattr__ = lambda attr: _Noop()
    for k, v in attrs.items():
        setattr(m, k, v)
    return m


def _hdf5_write(data, path=".", filename="out.h5", **kw):
    import numpy as np
    out = os.path.join(path, os.path.splitext(filename)[0] + ".npz")
    np.savez(out, **{k: np.asarray(v) for k, v in data.items()})


def install_stand_ins():
    """Headless stand-ins for matplotlib / h5py / hdf5storage where absent."""
    try:
        importlib.import_module("matplotlib")
    except ImportError:
        plt = _stub_module("matplotlib.pyplot")
        colors = _stub_module("matplotlib.colors")
        mpl = _stub_module("matplotlib", pyplot=plt, colors=colors, use=lambda *a, **k: None)
        sys.modules.update({"matplotlib": mpl, "matplotlib.pyplot": plt, "matplotlib.colors": colors})
    for name, attrs in (("h5py", {}), ("hdf5storage", {"write": _hdf5_write})):
        try:
            importlib.import_module(name)
        except ImportError:
            sys.modules[name] = _stub_module(name, **attrs)


def _sub(src, old, new, what, count=None, regex=False):
    n = len(re.findall(old, src)) if regex else src.count(old)
    if n == 0 or (count is not None and n != count):
        raise RuntimeError(f"driver patch '{what}': expected text not found ({n} matches)")
    return re.sub(old, new, src) if regex else src.replace(old, new)


def patch_source(src, name, keep_quirks=False, gpu_tables=False):
    """Apply the compatibility patches to a driver's source text."""
    src = _sub(src, "configparser.SafeConfigParser()", "configparser.ConfigParser()",
               "SafeConfigParser removed in Python 3.12")
    if name == "lookup.py":
        src = _sub(src, "np.float(", "float(", "np.float removed in numpy 1.24")
        src = _sub(src, "np.Inf", "np.inf", "np.Inf removed in numpy 2")
        if not keep_quirks:
            src = _sub(src, "mu_s__start*mu_a_base**i", "mu_s__start*mu_s__base**i",
                       "mu_s' axis built with mu_a_base", count=1)
        if gpu_tables:
            src = _sub(src, "def makelookup(", "def _reference_makelookup(", "makelookup", count=1)
    elif name == "minimization.py":
        if not keep_quirks:
            src = _sub(src, r"(M_U_unc'\)\.split\(\"\\n\"\),dtype=float\)\[0\][^\n]*\nelse:\n\s*)"
                            r"T_u_exact = None", r"\1T_u_exact_unc = None",
                       "T_u_exact_unc default", count=1, regex=True)
    return src


def gpu_makelookup(R_d, T_d, R_d_std, T_d_std, N, uncertainty=True, M=100, method="cubic",
                   graph=False, **filenames):
    """lookup.py:301 makelookup's signature and return values on the GPU path.
    The grid axes come from the driver's globals (mu_a, mu_s_), as they do in
    the driver's own function."""
    import numpy as np
    from ismc_gb300.lookup import make_lookup
    g = gpu_makelookup.driver_globals
    mua_t, ua, mus_t, us, Rv, Tv = make_lookup(R_d, T_d, R_d_std, T_d_std, g["mu_a"], g["mu_s_"],
                                               N=N, uncertainty=uncertainty, M=M)
    # the (R, T) sample points in percent, sorted by R then T (lookup.py:320-329)
    R_d, T_d = np.asarray(R_d, float), np.asarray(T_d, float)
    pts = np.stack([100 * R_d[1:, 1:].ravel(), 100 * T_d[1:, 1:].ravel()], 1)
    pts = pts[np.lexsort((pts[:, 1], pts[:, 0]))]
    return mua_t, ua, mus_t, us, Rv, Tv, pts, pts.copy()


def run_driver(path, argv, keep_quirks=False, gpu_tables=False, numpy_seed=None, ismc_seed=None):
    path = os.path.abspath(path)
    name = os.path.basename(path)
    if name not in ("lookup.py", "minimization.py"):
        raise ValueError(f"unknown driver {name}: expected lookup.py or minimization.py")
    with open(path) as f:
        src = f.read()
    src = patch_source(src, name, keep_quirks, gpu_tables)
    install_stand_ins()
    sys.path.insert(0, HERE)                    # our ISMC.py / ISMLMC.py first
    sys.argv = [path] + list(argv)
    os.chdir(os.path.dirname(path))
    g = {"__name__": "__main__", "__file__": path, "__builtins__": __builtins__}
    if gpu_tables:
        gpu_makelookup.driver_globals = g
        g["makelookup"] = gpu_makelookup
    # reproducible runs: the drivers draw their input distributions from
    # numpy's global generator, and the drop-in ISMC's k-th call uses Philox
    # stream k of its seed
    if numpy_seed is not None:
        import numpy as np
        np.random.seed(int(numpy_seed))
    if ismc_seed is not None:
        from ismc_gb300.dropin import _common
        _common.seed(int(ismc_seed))
    with warnings.catch_warnings():          # the drivers' "\m" in plot labels
        warnings.simplefilter("ignore", SyntaxWarning)
        code = compile(src, path, "exec")
    exec(code, g)
    return g


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("driver", help="path to lookup.py or minimization.py")
    ap.add_argument("--keep-quirks", action="store_true",
                    help="do not fix the two driver bugs (T_u_exact_unc, mu_s' axis base)")
    ap.add_argument("--gpu-tables", action="store_true",
                    help="lookup.py: build the tables with the GPU make_lookup")
    ap.add_argument("--numpy-seed", type=int, default=None,
                    help="seed numpy's global generator before the driver runs")
    ap.add_argument("--ismc-seed", type=int, default=None,
                    help="seed of the drop-in ISMC's call sequence")
    a, rest = ap.parse_known_args(argv)
    run_driver(a.driver, rest, a.keep_quirks, a.gpu_tables, a.numpy_seed, a.ismc_seed)


if __name__ == "__main__":
    main()
