"""GPU voxelizer: bit-identical to the reference's labelPoints."""
import numpy as np
import pytest

from helpers import fixtures, golden_mask, load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("path", fixtures("vox"), ids=lambda p: p.split("/")[-1])
def test_gpu_mask_matches_reference_golden(gpu_lib, path):
    d = load(path)
    mask, desc = gpu_lib.voxelize(d["tri12"], float(d["spacing"]))
    assert tuple(desc.dims) == tuple(d["dims"])
    assert np.array_equal(np.array(desc.bbox[:]), d["bbox"])
    assert desc.fluid_count == int(d["nfluid"])
    assert np.array_equal(mask, golden_mask(d))


def _random_soup(rng, n, scale=10.0):
    v = rng.uniform(0, scale, size=(n, 3, 3))
    # snap a third of the vertices to the lattice so rays meet edges/vertices exactly
    snap = rng.random((n, 3)) < 0.33
    v[snap] = np.round(v[snap])
    nrm = np.cross(v[:, 1] - v[:, 0], v[:, 2] - v[:, 0])
    ln = np.linalg.norm(nrm, axis=1, keepdims=True)
    ln[ln == 0] = 1
    nrm = nrm / ln
    # some facets carry a sloppy file normal, as real STL exports do
    bad = rng.random(n) < 0.2
    nrm[bad] = np.round(nrm[bad], 2)
    # degenerate facets
    v[:3, 2] = v[:3, 1]
    return np.concatenate([v.reshape(n, 9), nrm], axis=1)


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_gpu_mask_matches_oracle_on_random_soups(gpu_lib, oracle_lib, seed):
    """Brute-force oracle (every triangle for every point) vs the binned GPU
    kernel on adversarial soups: degenerate, lattice-snapped and steep facets."""
    rng = np.random.default_rng(seed)
    tri = _random_soup(rng, 300)
    for sp in (1.0, 0.5):
        ref, _, _ = oracle_lib.voxelize(tri, sp, culled=False)
        got, _ = gpu_lib.voxelize(tri, sp)
        assert np.array_equal(got, ref)


def test_gpu_mask_explicit_lattice(gpu_lib, oracle_lib):
    d = load(fixtures("vox")[0])
    tri = d["tri12"]
    bb = d["bbox"]
    org = (bb[0] - 2.0, bb[2] - 1.0, bb[4] - 3.0)
    dims = (30, 28, 110)
    ref, _, _ = oracle_lib.voxelize(tri, 1.0, bbox=bb, origin=org, dims=dims, culled=False)
    got, _ = gpu_lib.voxelize(tri, 1.0, bbox=bb, origin=org, dims=dims)
    assert np.array_equal(got, ref)


def test_gpu_mask_c2_bifurcation_full_size(gpu_lib, oracle_lib):
    """The 256x192x512 benchmark lattice: GPU mask == binned oracle mask
    (the binned oracle is pinned to the brute force and the reference above)."""
    from pv_dec_original_gb300 import geometry as G
    tri = G.config_c2_bifurcation().tri12()
    got, desc = gpu_lib.voxelize(tri, 1.0)
    assert tuple(desc.dims) == (256, 192, 512)
    ref, _, _ = oracle_lib.voxelize(tri, 1.0, culled=True, nthreads=0)
    assert np.array_equal(got, ref)
