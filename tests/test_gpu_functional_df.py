"""The double-float closed-shell functional of the tensor-core quadrature against the FP64 form.

Both run on the device through calchem_xc_eval_closed_shell: precision FP64 is the FP64
quadrature's xc_eval_cs (CalChem's eval_xc_spin at rho_a = rho_b, crates/calchem-dft/src/xc.rs:159),
precision MIXED the form the tensor-core kernels use (double-float arithmetic on the FP32 pipe for
SVWN5..PBE0 at total density >= 1e-12, FP64 below and for the range-separated codes).
"""

import numpy as np
import pytest

from calchem_gb300 import eval_closed_shell_gpu

pytestmark = pytest.mark.gpu

CODES_DF = ["svwn5", "blyp", "pbe", "b3lyp", "b3lyp5", "pbe0"]
# Agreement of the two forms, relative to the energy-density scale of each output: ~1e-14 typical,
# a few 1e-10 where the exchange and correlation terms of f cancel to a few digits.
TOL = 1e-9


def _sweep():
    """Spin densities 1e-13..1e4 (total 2e-13..2e4) times reduced gradients s = 0..1e3
    (|grad rho_a| = s 2 (3 pi^2)^(1/3) rho_a^(4/3), gamma = |grad rho_a|^2)."""
    r = np.logspace(-13, 4, 341)
    s = np.concatenate([[0.0], np.logspace(-4, 3, 29)])
    R, S = np.meshgrid(r, s, indexing="ij")
    grad = S * 2.0 * (3.0 * np.pi ** 2) ** (1.0 / 3.0) * R ** (4.0 / 3.0)
    return R.ravel(), (grad * grad).ravel()


@pytest.mark.parametrize("name", CODES_DF)
def test_double_float_functional_matches_fp64(name):
    r, g = _sweep()
    ref = eval_closed_shell_gpu(name, r, g, precision="fp64")
    got = eval_closed_shell_gpu(name, r, g, precision="mixed")
    assert np.all(np.isfinite(got))
    f, vr, vg = ref[:, 0], ref[:, 1], ref[:, 2]
    scale_f = np.abs(f)
    scale_r = np.abs(f) + np.abs(vr) * r
    scale_g = np.abs(f) + np.abs(vg) * g
    live = 2 * r >= 1e-12
    err_f = np.abs(got[:, 0] - f) / np.where(scale_f > 0, scale_f, 1.0)
    err_r = np.abs(got[:, 1] - vr) * r / np.where(scale_r > 0, scale_r, 1.0)
    err_g = np.abs(got[:, 2] - vg) * g / np.where(scale_g > 0, scale_g, 1.0)
    worst = max(err_f[live].max(), err_r[live].max(), err_g[live].max())
    assert worst < TOL, (name, err_f[live].max(), err_r[live].max(), err_g[live].max())
    # below the double-float range the FP64 form itself runs: identical results
    assert np.array_equal(got[~live], ref[~live])


@pytest.mark.parametrize("name", ["cam-b3lyp", "wb97x", "wb97x-d"])
def test_range_separated_codes_keep_fp64(name):
    r, g = _sweep()
    assert np.array_equal(eval_closed_shell_gpu(name, r, g, precision="mixed"),
                          eval_closed_shell_gpu(name, r, g, precision="fp64"))

