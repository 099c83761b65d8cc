"""Host-side set-up of the product against the oracle, and the C ABI surface.

The block-tree neighbour lists, the Yin-Yang interpolation coordinates and the
ghost maps must be bit-identical to the reference's (restated by the oracle).
These run without a GPU: falcon_create with device=-1 builds the host side only.
"""
import ctypes as C
import os
import re

import numpy as np
import pytest

import falcon_gb300 as fg
import oracle
from falcon_gb300 import config

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def _built(built_lib):
    return built_lib


def test_library_exports_every_declared_symbol():
    hdr = open(os.path.join(ROOT, "include", "falcon_gb300.h")).read()
    declared = set(re.findall(r"\b(falcon_[a-z0-9_]+)\s*\(", hdr))
    assert declared == set(fg.EXPORTS)
    L = C.CDLL(fg.LIB_PATH)
    for name in declared:
        assert hasattr(L, name), name


@pytest.mark.parametrize("mk", [config.tiny, config.shell_fp64_cpu])
def test_tree_geometry_background_bit_identical(mk):
    f = fg.Falcon(mk(device=-1))
    o = oracle.Oracle(mk())
    assert (f.nblocks, f.nblocks_yin) == (o.nblocks, o.nblocks_yin)
    assert np.array_equal(f.block_ranges(), o.block_ranges())
    assert np.array_equal(f.block_flags(), o.block_flags())
    assert np.array_equal(f.background(), o.background())


@pytest.mark.parametrize("mk", [config.tiny, config.shell_fp64_cpu])
def test_ghost_map_bit_identical(mk):
    f = fg.Falcon(mk(device=-1))
    o = oracle.Oracle(mk())
    a, b = f.ghost_map(), o.ghost_map()
    assert len(a) == len(b) == o.ghost_count()
    assert a.tobytes() == b.tobytes()
    assert o.uncovered_ghosts() == 0


def test_reference_tree_without_root_tiling_and_geometric_radial():
    """root_tiles=(1,1,1) is the reference tree itself (PARAM.in-style
    #RADIALGRID + #AMR), here with the geometric radial rule (option 3)."""
    mk = lambda **kw: config.make_config(block=(8, 8, 8), root_tiles=(1, 1, 1), radial_levels=2,
                                         radial_option=3, amr=((0, 1, 1), (0, 1, 1)), **kw)
    f = fg.Falcon(mk(device=-1))
    o = oracle.Oracle(mk())
    assert np.array_equal(f.block_ranges(), o.block_ranges())
    assert f.ghost_map().tobytes() == o.ghost_map().tobytes()


def test_block_counts_of_the_workloads():
    assert fg.Falcon(config.shell_fp64_cpu(device=-1)).nblocks == 864
    f = fg.Falcon(config.shell_mixed_21m(device=-1))
    assert f.nblocks == 5184 and f.interior_cells == 21233664


def test_invalid_configs_fail_loudly():
    with pytest.raises(fg.FalconError) as e:
        fg.Falcon(config.tiny(device=-1, ng=3))
    assert e.value.code == fg.ERR_INVALID_ARG
    with pytest.raises(fg.FalconError):
        fg.Falcon(config.tiny(device=-1, cfl=-1.0))
    with pytest.raises(fg.FalconError):
        fg.Falcon(config.tiny(device=-1, if_involve_B=0))
    with pytest.raises(fg.FalconError):
        fg.Falcon(config.tiny(device=-1, divb_option=3))
    with pytest.raises(fg.FalconError):
        fg.Falcon(config.tiny(device=-1, divb_option=1, if_involve_B=0))
    for d in (1, 2):
        fg.Falcon(config.tiny(device=-1, divb_option=d)).close()


def test_device_calls_without_device_are_errors():
    f = fg.Falcon(config.tiny(device=-1))
    with pytest.raises(fg.FalconError) as e:
        f.advance_rk4()
    assert e.value.code == fg.ERR_NO_DEVICE
