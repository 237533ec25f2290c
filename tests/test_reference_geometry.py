"""The reference's serpentine geometry fixture (tests/golden/domain_snake_420_180.npz): the raw
values of microfluidics_complex_domain/domain_snake_420_180.bin and _dist.bin, checked against
the files themselves where the reference tree is present, and the README example built on it."""
import os

import numpy as np
import pytest

from drd_application_gb300 import abi
from drd_application_gb300.workloads import load_reference_geometry, make_reference_snake, mask_cell
from tests.golden import make_reference_geometry as mrg

GEOM = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "domain_snake_420_180.npz")
REF = os.path.join("/root/reference", "microfluidics_complex_domain")


def test_fixture_values():
    mask, dist = load_reference_geometry(GEOM)
    assert mask.shape == dist.shape == (180, 420)
    assert set(np.unique(mask)) == {-1.0, 1.0}
    assert 0.0 <= dist.min() and dist.max() < 0.2502
    # the channel: walls (mask 1) at the top and bottom of every column, fluid between
    assert np.all(mask[0] == 1.0) and np.all(mask[-1] == 1.0) and (mask == -1.0).mean() > 0.3


@pytest.mark.skipif(not os.path.isdir(REF), reason="reference tree not present")
def test_fixture_equals_reference_files():
    z = np.load(GEOM)
    for key, fname in mrg.FILES.items():
        assert np.array_equal(z[key], mrg.read_var(os.path.join(REF, fname)))


def test_reference_snake_case():
    mask, dist = load_reference_geometry(GEOM)
    m = mask_cell(mask)
    bdr = np.clip((m + 1.0) / 2.0, 0.0, 1.0)
    case = make_reference_snake(bdr, dist)
    P = case.params
    assert (P.nr, P.nz) == (420, 180) and P.lambda_eta == 100.0 and P.two_fluid == 0
    ph = case.state[abi.F_PH]
    assert ph.min() >= 0.0 and ph.max() <= 1.0 and np.all(ph <= 1.0 - bdr + 1e-15)
    pts = case.meta["particles"]["points"]
    assert pts.shape == (2, 9) and abs(pts[0].mean() - 1.75) < 1e-12 and abs(pts[1].mean() - 0.42) < 1e-12
