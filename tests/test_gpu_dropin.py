"""The drop-in modules keep the reference's call surface (ISMC.py:164-165,
ISMLMC.py:101-102) and statistics."""

import pytest

import cases

pytestmark = pytest.mark.gpu


def _args(c):
    s = c["spheres"]
    return (s["R"], s["R_pw"], s["R_fs"], s["R_fp"], s["R_fd"], s["R_f"], s["R_angle"],
            s["specular_included"], s["T"], s["T_pw"], s["T_fs"], s["T_fp"], s["T_fd"], s["T_f"],
            s["T_angle"])


def test_dropin_ismc_signature_and_statistics(engine):
    from ismc_gb300.dropin import ISMC as M
    c = cases.golden()["ismc_example"]
    L = c["layers"][0]
    N = 2_000_000
    out = M.ISMC(N, L["n"], L["g"], L["d"], L["mua"], L["mus"], L["mua"] + L["mus"], *_args(c))
    assert isinstance(out, tuple) and len(out) == 5
    means, se, status = M.ISMC_ex(N, L["n"], L["g"], L["d"], L["mua"], L["mus"],
                                  L["mua"] + L["mus"], *_args(c), seed=5)
    assert status == 0
    z = cases.zscores(means, se, c["mean"], c["se"])
    assert max(abs(x) for x in z) <= 4.0, z
    # calls draw distinct streams (like successive calls on the global RNG)
    out2 = M.ISMC(N, L["n"], L["g"], L["d"], L["mua"], L["mus"], L["mua"] + L["mus"], *_args(c))
    assert out != out2


def test_dropin_ismlmc_lists_and_int_flags(engine):
    from ismc_gb300.dropin import ISMLMC as M
    c = cases.golden()["bench0_slides"]
    Ls = c["layers"]
    col = lambda k: [L[k] for L in Ls]
    mut = [L["mua"] + L["mus"] for L in Ls]
    args = list(_args(c))
    args[0], args[8] = 1, 1          # callers pass 0/1 ints (minimization.py:100)
    means, se, status = M.ISMLMC_ex(2_000_000, col("n"), col("g"), col("d"), col("mua"),
                                    col("mus"), mut, *args, seed=8)
    z = cases.zscores(means, se, c["mean"], c["se"])
    assert status == 0 and max(abs(x) for x in z) <= 3.0, z
    with pytest.raises(ValueError):
        M.ISMLMC(10, col("n"), col("g")[:2], col("d"), col("mua"), col("mus"), mut, *args)
