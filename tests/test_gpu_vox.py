"""GPU casts on scenes imported from .vox files (svo_scene_from_vox): the device image of an imported
scene casts like the oracle's tree built by the oracle's importer (oracle/vox.py), every field and
counter."""
import numpy as np
import pytest

import shocovox_gb300 as svo
from oracle import vox as V
from test_gpu_cast import assert_same_hits, random_rays
from vox_writer import random_scene

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("rotate,dim", [(False, 2), (True, 1), (True, 4)])
def test_imported_scene_casts_like_the_oracle(oracle_mod, rotate, dim):
    done = 0
    for seed in range(40):
        data = random_scene(np.random.default_rng(500 + seed), n_models=5, max_size=40, rotate=rotate)
        try:
            o = V.build(oracle_mod, data, dim)
        except V.VoxPanic:  # voxels the reference's bounds put outside the octree
            continue
        p = svo.Octree.from_vox(data, dim)
        p.upload()
        origins, dirs = random_rays(np.random.default_rng(seed), p.size, 3000)
        assert_same_hits(p.cast_host(origins, dirs), o.cast(origins, dirs, threads=8), counters=True,
                         label="vox seed %d" % seed)
        done += 1
        if done == 3:
            break
    assert done == 3
