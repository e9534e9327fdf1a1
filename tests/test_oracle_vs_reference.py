"""The oracle against the reference's own code (oracle/_ref, compiled from
the reference sources by oracle/build_ref.sh where they are present) on
parameter sets beyond the golden fixtures: wider search windows, more
matches per frame, larger groups, fewer frames searched, a denser grid.
Bit-exact, like the golden tests.  Skipped where the reference library has
not been built."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle, RefLib
from vbm3d_gb300._abi import dims_of
from vbm3d_gb300.synth import make_clip

pytestmark = pytest.mark.skipif(not RefLib.available(exact=True), reason="reference library not built")

# (channels, sigma, colour transform, flows, step-1 and step-2 overrides)
CASES = [
    (1, 20.0, False, True, dict(Ns=11, Npr=9)),
    (3, 20.0, True, False, dict(Ns=11, Npr=9)),
    (1, 10.0, False, False, dict(Nb=3, N=16)),
    (3, 30.0, True, True, dict(Ns=9, Npr=7, Nb=4, Nf=2)),
    (1, 50.0, False, True, {}),
    (3, 25.0, False, False, dict(p=2)),
]


@pytest.fixture(scope="module")
def libs():
    return Oracle(), RefLib(exact=True)


@pytest.mark.parametrize("case", range(len(CASES)))
def test_matches_reference(libs, case):
    o, r = libs
    c, sigma, cs, flows, over = CASES[case]
    _, noisy, ff, bf = make_clip(44, 36, 6, c, sigma, 600 + case, with_flow=flows)
    p1 = o.default_params(1, sigma).replace(**over)
    p2 = o.default_params(2, sigma).replace(**over)
    vid = o.color_transform(noisy, True) if cs else noisy
    for p in (p1, p2):
        pidx = o.ref_indices(p, dims_of(vid))
        got, want = o.similar(p, vid, ff, bf), r.similar(p, vid, pidx, ff, bf)
        for key in ("idx", "dist", "nsimp", "nsx"):
            np.testing.assert_array_equal(got[key], want[key], err_msg=key)
    gb, gf = o.run(sigma, noisy, p1, p2, ff, bf, cs, threads=1)
    wb, wf = r.run(sigma, noisy, p1, p2, ff, bf, color_space=cs, threads=1)
    np.testing.assert_array_equal(gb, wb)
    np.testing.assert_array_equal(gf, wf)
