import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GB300 (sm_103a) device")


@pytest.fixture(scope="session", autouse=True)
def _built():
    """Builds (incrementally) the CUDA library and the CPU oracle once."""
    from kagayaki_gb300 import build as kb
    kb.build()
    from oracle import orc
    orc.build()
    yield


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


C1_LO, C1_HI = (-4.99, 0.01, -4.99), (4.99, 9.99, 4.99)


def sample_stats(ours, ref, tol=1e-4):
    """Per-sample agreement of (frames, pixels, 3) compat samples with the
    reference's (pixel 0 dropped: its seed divides by zero in the
    reference).  identical: bit for bit; close: within `tol` relative;
    close_frame0: the same in the first frame (no seed chain behind it);
    chains_in_step: pixels whose every frame stayed close (a flipped
    decision puts a pixel's seed chain out of step for the frames after)."""
    a, b = ours[:, 1:], ref[:, 1:]
    rel = (np.abs(a - b) / np.maximum(np.abs(b), 1e-4)).max(-1)
    close = rel <= tol
    return dict(identical=float((a == b).all(-1).mean()), close=float(close.mean()),
                close_frame0=float(close[0].mean()), chains_in_step=float(close.all(0).mean()))


# Per-sample bars of the compat estimator against the reference's host build,
# set from measurements on the GB300 (C1 256x256x16 / Disney / textured /
# environment scenes): within 1e-4 relative 99.3-100 % of first-frame samples
# and 98.6-100 % of all samples; pixel chains in step 91 % after 16 frames,
# 95.6-99.8 % after 6.  Compiling the renderer with -fmad=false (the host
# build's rounding) raised these to 99.7 % / 97 %: FMA contraction explains
# about three quarters of the departures, CUDA's libm the rest.
BAR_CLOSE_FRAME0 = 0.985
BAR_CLOSE = 0.975
