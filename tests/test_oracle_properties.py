"""Properties of the oracle's physics mode that hold at any size.  The
reference has parity semantics only, so its golden fixtures pin the
oracle's parity mode; these pin the physics mode's streaming, half-way
bounce-back and collisions (BGK and regularized, D3Q19 and D3Q27): a
closed vessel conserves mass to round-off from any state, the rest state
is a fixed point, a mirror-symmetric vessel with a mirror-symmetric
state stays mirror-symmetric, Zou-He rules impose exactly the prescribed
inlet profile and outlet density, a steady tube carries the same mass
flux through every cross-section, and interpolated (Bouzidi) bounce-back
with every wall half a spacing away is half-way bounce-back bit for bit."""
import numpy as np
import pytest

from helpers import classify


def _vessel(shape=(14, 11, 9)):
    """A closed ellipsoidal cavity, cls[k, j, i] (1 fluid, 0 solid),
    symmetric under i -> nx - 1 - i."""
    nz, ny, nx = shape
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cz, cy, cx = (nz - 1) / 2, (ny - 1) / 2 + 0.3, (nx - 1) / 2
    r = ((k - cz) / (0.45 * nz)) ** 2 + ((j - cy) / (0.42 * ny)) ** 2 + ((i - cx) / (0.44 * nx)) ** 2
    return (r < 1.0).astype(np.uint8)


def _sim(O, Q, regularized, cls, tau=0.7):
    s = O.Sim(Q, O.PHYSICS, cls, (0.0, 0.0, 0.0), 1.0, tau, [])
    s.set_collision(regularized)
    return s


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("regularized", [False, True])
def test_closed_vessel_conserves_mass(oracle_lib, Q, regularized):
    O = oracle_lib
    s = _sim(O, Q, regularized, _vessel())
    f, _, _ = s.f()
    rng = np.random.default_rng(Q + 10 * regularized)
    s.set_f(f * (1.0 + 0.02 * rng.uniform(-1.0, 1.0, size=f.shape)))
    m0, _, _ = s.conservation()
    s.step(60)
    m1, _, _ = s.conservation()
    assert abs(m1 - m0) <= 1e-12 * abs(m0), (m0, m1)
    rho, u = s.macro()
    assert np.all(np.isfinite(rho)) and np.abs(u).max() < 0.1


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("regularized", [False, True])
def test_rest_state_is_a_fixed_point(oracle_lib, Q, regularized):
    O = oracle_lib
    s = _sim(O, Q, regularized, _vessel())
    f0, _, _ = s.f()
    s.step(25)
    f1, _, _ = s.f()
    assert np.abs(f1 - f0).max() <= 1e-15
    _, u = s.macro()
    assert np.abs(u).max() <= 1e-15


@pytest.mark.parametrize("Q", [19, 27])
def test_mirror_symmetry_is_kept(oracle_lib, Q):
    """Mirror i -> nx - 1 - i maps population q to the one with c_x negated;
    a state built symmetric stays symmetric (to round-off) in a symmetric
    cavity."""
    O = oracle_lib
    cls = _vessel()
    assert np.array_equal(cls, cls[:, :, ::-1])
    s = _sim(O, Q, False, cls)
    c, _, _ = O.lattice(Q)
    c = np.asarray(c)
    mirror_q = np.array([int(np.where((c[:, 0] == -c[q, 0]) & (c[:, 1] == c[q, 1]) & (c[:, 2] == c[q, 2]))[0][0])
                         for q in range(Q)])
    pt, _ = s.active()
    nz, ny, nx = cls.shape
    i, j, k = pt % nx, (pt // nx) % ny, pt // (nx * ny)
    index = {int(p): a for a, p in enumerate(pt)}
    partner = np.array([index[int((kk * ny + jj) * nx + (nx - 1 - ii))] for ii, jj, kk in zip(i, j, k)])
    f, _, _ = s.f()
    rng = np.random.default_rng(Q)
    g = f * (1.0 + 0.02 * rng.uniform(-1.0, 1.0, size=f.shape))
    g = 0.5 * (g + g[partner][:, mirror_q])  # symmetrise
    s.set_f(g)
    s.step(40)
    h, _, _ = s.f()
    assert np.abs(h - h[partner][:, mirror_q]).max() <= 1e-14


def _tube(O, Q, regularized, u_in=0.02, tau=0.8):
    """Capped z tube (radius 4.3 in a 12 x 12 section, 38 planes), parabolic
    velocity inlet on its first fluid plane, density 1 outlet on its last."""
    nz, ny, nx = 40, 12, 12
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    mask = (((i - 5.5) ** 2 + (j - 5.5) ** 2) < 4.3 ** 2).astype(np.uint8)
    mask[0] = 0
    mask[-1] = 0
    fl = np.argwhere(mask > 0)
    kin, kout = int(fl[:, 0].min()), int(fl[:, 0].max())
    cls = classify(mask, [(2, kin), (2, kout)])
    bcs = [dict(kind=O.BC_VELOCITY, face=4, plane=kin, value=1.0, profile=1, c1=5.5, c2=5.5, R=4.3),
           dict(kind=O.BC_PRESSURE, face=5, plane=kout, value=1.0)]
    s = O.Sim(Q, O.PHYSICS, cls, (0.0, 0.0, 0.0), 1.0, tau, bcs)
    s.set_collision(regularized)
    s.set_amplitude([u_in])
    return s, (nx, ny), (kin, kout)


@pytest.mark.parametrize("Q", [19, 27])
@pytest.mark.parametrize("regularized", [False, True])
def test_zou_he_imposes_inlet_profile_and_outlet_density(oracle_lib, Q, regularized):
    O = oracle_lib
    s, (nx, ny), (kin, kout) = _tube(O, Q, regularized)
    s.step(300)
    pt, c = s.active()
    k, j, i = pt // (nx * ny), (pt // nx) % ny, pt % nx
    rho, u = s.macro()
    inlet = (c >= 3) & (k == kin)
    outlet = (c >= 3) & (k == kout)
    assert inlet.sum() > 40 and outlet.sum() > 40
    want = 0.02 * (1.0 - ((i[inlet] - 5.5) ** 2 + (j[inlet] - 5.5) ** 2) / 4.3 ** 2)
    assert np.abs(u[inlet, 2] - want).max() <= 1e-15
    assert np.abs(u[inlet, :2]).max() <= 1e-15
    assert np.abs(rho[outlet] - 1.0).max() <= 1e-15


def test_steady_tube_carries_one_mass_flux(oracle_lib):
    """After the start-up transient has decayed, sum(rho u_z) over each
    cross-section agrees along the tube (0.23% apart after 2000 steps,
    0.03% after 16000)."""
    O = oracle_lib
    s, (nx, ny), (kin, kout) = _tube(O, 19, False)
    s.step(12000)
    pt, _ = s.active()
    k = pt // (nx * ny)
    rho, u = s.macro()
    flux = np.array([(rho[k == z] * u[k == z, 2]).sum() for z in range(kin, kout + 1)])
    assert (flux.max() - flux.min()) / flux.mean() < 1e-3, flux


def _box_triangles(lo, hi):
    """The 12 outward-facing triangles of an axis-aligned box, tri12 rows
    (three vertices, then the unit normal)."""
    (x0, y0, z0), (x1, y1, z1) = lo, hi
    v = np.array([[x0, y0, z0], [x1, y0, z0], [x1, y1, z0], [x0, y1, z0],
                  [x0, y0, z1], [x1, y0, z1], [x1, y1, z1], [x0, y1, z1]], np.float64)
    faces = [(0, 2, 1), (0, 3, 2), (4, 5, 6), (4, 6, 7), (0, 1, 5), (0, 5, 4),
             (3, 7, 6), (3, 6, 2), (0, 4, 7), (0, 7, 3), (1, 2, 6), (1, 6, 5)]
    rows = []
    for a, b, c in faces:
        n = np.cross(v[b] - v[a], v[c] - v[a])
        rows.append(np.concatenate([v[a], v[b], v[c], n / np.linalg.norm(n)]))
    return np.array(rows)


@pytest.mark.parametrize("Q", [19, 27])
def test_interpolated_walls_at_half_spacing_are_half_way(oracle_lib, Q):
    """A box cavity whose walls lie half a spacing outside its outer nodes:
    every missing link has q = 1/2 and the Bouzidi rule reduces to half-way
    bounce-back exactly; walls a quarter spacing away change the flow."""
    O = oracle_lib
    nz, ny, nx = 9, 8, 7
    cls = np.zeros((nz + 2, ny + 2, nx + 2), np.uint8)
    cls[1:-1, 1:-1, 1:-1] = 1
    half = O.Sim(Q, O.PHYSICS, cls, (0.0, 0.0, 0.0), 1.0, 0.7, [])
    bouzidi = O.Sim(Q, O.PHYSICS, cls, (0.0, 0.0, 0.0), 1.0, 0.7, [])
    bouzidi.set_wall_distances(_box_triangles((0.5, 0.5, 0.5), (nx + 0.5, ny + 0.5, nz + 0.5)))
    assert np.array_equal(np.unique(bouzidi.wall_distances()), [0.5])
    quarter = O.Sim(Q, O.PHYSICS, cls, (0.0, 0.0, 0.0), 1.0, 0.7, [])
    quarter.set_wall_distances(_box_triangles((0.75, 0.75, 0.75), (nx + 0.25, ny + 0.25, nz + 0.25)))
    assert 0.25 in np.unique(quarter.wall_distances())
    f, _, _ = half.f()
    g = f * (1.0 + 0.02 * np.random.default_rng(Q).uniform(-1.0, 1.0, size=f.shape))
    for s in (half, bouzidi, quarter):
        s.set_f(g)
        s.step(30)
    fh, fb, fq = half.f()[0], bouzidi.f()[0], quarter.f()[0]
    assert np.array_equal(fh, fb)
    assert np.abs(fq - fh).max() > 1e-6
