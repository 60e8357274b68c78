"""The seeded box dielectric of the 3D 256^3 configuration against the
reference's own rasteriser: ``Box.contains`` / ``GeometryGroup.rasterize``
(geometry/shapes.py:71-132, 338-376) evaluated at the cell centres, painted in
draw order, must give the identical eps array that ``workloads.boxes_3d``
builds (CPU, full size)."""

import numpy as np
import pytest

from helpers import SOURCE_TREES, import_reference


def _reference_eps(prismo, dims, dx, specs, background):
    from prismo.geometry.shapes import Box, GeometryGroup, Material

    boxes = [Box(Material(f"box{q}", epsilon_r=float(v)), tuple(np.asarray(c) * dx), tuple(np.asarray(e) * dx))
             for q, (c, e, v) in enumerate(specs)]
    axes = [(np.arange(n) + 0.5) * dx for n in dims]
    combined, masks = GeometryGroup(boxes, "union").rasterize(*axes)
    eps = np.full(dims, float(background))
    for b, m in zip(boxes, masks):  # later shapes overwrite earlier ones
        eps[m] = b.material.epsilon_r
    return eps, combined


@pytest.mark.parametrize("dims,dx", [((256, 256, 256), 20e-9), ((96, 80, 64), 1.0)])
def test_boxes_3d_equals_reference_rasteriser(dims, dx):
    prismo = import_reference(SOURCE_TREES)  # skips without the reference package
    from prismo_gb300.workloads import CONFIG_3D, EPS_SIO2, box_specs_3d, boxes_3d

    seed = CONFIG_3D["seed"]
    specs = box_specs_3d(dims, nboxes=CONFIG_3D["nboxes"], seed=seed)
    want, combined = _reference_eps(prismo, dims, dx, specs, EPS_SIO2)
    got = boxes_3d(dims, nboxes=CONFIG_3D["nboxes"], seed=seed)
    assert combined.any() and not combined.all()
    assert np.array_equal(got, want), int((got != want).sum())
