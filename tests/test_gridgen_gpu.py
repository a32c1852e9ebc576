"""The device grid build (lbm_grid_create_device) against the host build.

The device enumerates the curve indices of the level in order and numbers the
kept cells with a prefix sum instead of sorting; with the same geometry code
on both sides the tables must be equal bit for bit: on every fixture's config
(2D and 1D, stretched grids and the obstacle case included) and on 3D
configurations that the reference cannot build.
"""
import json
import os

import numpy as np
import pytest

import caseio
from helpers import channel_sphere_config
from lbm_gb300 import gridgen

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))
CONFIGS = json.load(open(os.path.join(HERE, "golden", "grid_configs.json")))


def same_tables(a, b):
    assert np.array_equal(a.centers, b.centers)
    assert np.array_equal(a.nghbr, b.nghbr)
    assert a.cell_length == b.cell_length and np.array_equal(a.bbox, b.bbox)
    assert sorted(a.surfaces) == sorted(b.surfaces)
    for k in a.surfaces:
        assert np.array_equal(a.surfaces[k]["cells"], b.surfaces[k]["cells"]), k
        assert np.array_equal(a.surfaces[k]["normals"], b.surfaces[k]["normals"]), k


@pytest.mark.parametrize("case", sorted(CONFIGS))
def test_device_build_equals_host_build(case):
    cfg = CONFIGS[case]
    same_tables(gridgen.grid_tables(cfg, device=0), gridgen.grid_tables(cfg))


def test_device_build_equals_the_reference_fixture():
    _, _, ref, _ = caseio.load("sphere_ns_l5_60")
    same_tables(gridgen.grid_tables(CONFIGS["sphere_ns_l5"], device=0), ref)


@pytest.mark.parametrize("level,radius", [(5, 3.0), (6, 5.5)])
def test_device_build_3d(level, radius):
    cfg = channel_sphere_config(level=level, radius=radius)
    same_tables(gridgen.grid_tables(cfg, device=0), gridgen.grid_tables(cfg))


def test_device_build_many_spheres_3d():
    """Several bodies and many subtracted spheres (the Poisson-Boltzmann
    configuration's geometry), one of them cut by the box."""
    rng = np.random.default_rng(5)
    geom = {"box": {"type": "box", "A": [0.0, 0.0, 0.0], "B": [64.0, 64.0, 64.0], "body": "fluid"}}
    for i in range(12):
        geom[f"s{i:02d}"] = {"type": "sphere", "center": rng.uniform(4, 60, 3).tolist(), "radius": float(rng.uniform(2, 6)),
                             "body": "fluid", "subtract": True}
    geom["s99"] = {"type": "sphere", "center": [0.0, 32.0, 32.0], "radius": 5.0, "body": "fluid", "subtract": True}
    cfg = {"dim": 3, "partitionLevel": 6, "uniformLevel": 6, "maxRfnmtLvl": 6, "geometry": geom,
           "solver": {"boundary": {"box": {"all": {"type": "wall"}}}}}
    same_tables(gridgen.grid_tables(cfg, device=0), gridgen.grid_tables(cfg))
