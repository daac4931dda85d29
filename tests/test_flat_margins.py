"""How far the flats' potentials are from flipping a receiver, on the oracle.

The facet rule reads the flats' potential, which the device solves with block reductions where the
reference sums in member order, so the device's potential may differ from the reference's in its
last bits (the routing tests bound it at 1e-12 relative). The receivers are bit-exact on every
world tested; this measures why, and how much room there is. A raised cell's laid value carries the
solver's rounding only when its flat has two or more members, the flat was laid, and the cell is not
the flat's unique highest member (laid at potential / highest = 1 exactly). For every land cell
beside such a value, oracle.facet_flip_delta gives the relative change of those values that could
change its receiver, to first order. That change can come through the gap between the winning facet
and one that sends the water to another cell, through the winning facet's slope against zero, or
through its diagonal share against the cell's Rho8 draw. On these worlds the smallest such change
is 1.5e-14 relative or more, about 70 units in the last place of a double: the device's potential
would have to be that far off at the deciding cells to flip a receiver.
"""
import numpy as np
import pytest

import oracle
from cartogenesis_gb300 import synthetic

ndimage = pytest.importorskip("scipy.ndimage")


def min_flip_delta(W, H, seed):
    h, _, _ = synthetic.world(W, H, seed)
    _, land, rel, _ = oracle.percentile_cut(h, 0.70, 0.0)
    filled = oracle.fill_depressions(land, rel)
    _, surf, _ = oracle.flow_directions(land, rel, filled, seed, 1.0, 214, want_surface=True)
    raised = (land == 1) & (filled > rel)
    lab, nl = ndimage.label(raised, structure=np.ones((3, 3)))
    sizes = np.bincount(lab.ravel())
    moving = raised & (sizes[lab] >= 2) & (surf != filled.astype(np.float64))
    top = ndimage.maximum(surf, labels=lab, index=np.arange(nl + 1))
    at_top = raised & (surf == top[lab])
    moving &= ~(at_top & (np.bincount(lab[at_top], minlength=nl + 1)[lab] == 1))
    near = np.zeros_like(moving)
    for dr in (-1, 0, 1):
        for dc in (-1, 0, 1):
            sh = np.roll(moving, dc, axis=1)
            if dr == 1:
                sh = np.vstack([np.zeros((1, W), bool), sh[:-1]])
            elif dr == -1:
                sh = np.vstack([sh[1:], np.zeros((1, W), bool)])
            near |= sh
    near &= land == 1
    d = oracle.facet_flip_delta(surf, near, moving, seed, 1.0)
    return int(near.sum()), float(d[np.isfinite(d)].min())


@pytest.mark.parametrize("W,H,seed", [(256, 128, 42), (512, 256, 7), (1024, 512, 3), (2048, 1024, 1)])
def test_no_receiver_beside_a_flat_flips_below_seventy_ulps(W, H, seed):
    cells, delta = min_flip_delta(W, H, seed)
    assert cells > 500
    assert delta >= 1.5e-14, delta
