"""Host-side bookkeeping of the ROM driver (pressio-demoapps_gb300/rom.py),
no GPU: the parameter designs and the fallback run's step / checkpoint
consistency."""
from __future__ import annotations

import importlib.util
import os

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def R():
    spec = importlib.util.spec_from_file_location("pda_gb300_rom", os.path.join(REPO, "pressio-demoapps_gb300",
                                                                                 "rom.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_latin_hypercube_has_one_point_per_stratum(R):
    pts = R.latin_hypercube(48, seed=5)
    assert len(pts) == 48
    for name, (lo, hi) in R.SWE_RANGES.items():
        v = np.array([p[name] for p in pts])
        assert np.all((v >= lo) & (v <= hi))
        strata = np.floor((v - lo) / (hi - lo) * 48).astype(int)
        assert sorted(np.minimum(strata, 47)) == list(range(48)), name


def test_fallback_run_rejects_checkpoints_off_the_rom_step_grid(R):
    # 100 FOM steps are not a whole number of ROM steps of 8 FOM steps: the
    # ROM state would be compared with the FOM state at another time
    with pytest.raises(ValueError, match="multiple"):
        R.FallbackRun(None, None, None, None, None, 0.005, 8, [100, 200, 300, 400], threshold=1.0)
