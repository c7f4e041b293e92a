"""The oracle's restatement of ansys::SoluteCluster on the CPU.

* GetEnergyOfCluster (EnergyPredictor.cpp:97-184) on the lattice, on the solute
  configuration of SoluteCluster::GetFormationEnergy and on the pure solvent equals
  the reference's own values (tests/golden/clusters_quaternary.npz, from the
  reference sources compiled by oracle/build_ref.sh) for 84 site lists: the
  oracle's clusters of the case, single solute sites and a vacancy.
* GetChemicalPotential (EnergyPredictor.cpp:196-214) from the oracle's census
  equals the reference's.
* The cluster search (SoluteCluster.cpp:277-373) equals an independent
  breadth-first restatement written here over the oracle's neighbour lists."""
from collections import deque

import numpy as np
import pytest

from latticemontecarlo_gb300 import synthetic as S

from tests.golden.make_golden import case_inputs


@pytest.fixture(scope="module")
def case(oracle_mod):
    elements, coeffs, n, species = case_inputs("clusters_quaternary")
    g = np.load("tests/golden/clusters_quaternary.npz")
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(elements, coeffs, lat)
    return elements, coeffs, n, species, g, lat, m


def test_cluster_energies_match_reference(oracle_mod, case):
    elements, coeffs, n, species, g, lat, m = case
    solvent = S.alphabet(elements).index("Al")
    off, mem, ref = g["offsets"], g["members"], g["energies"]
    assert len(off) - 1 == ref.shape[0] == 84
    for k in range(ref.shape[0]):
        ids = mem[off[k]:off[k + 1]]
        got = [oracle_mod.cluster_energy(m, lat, species, solvent, ids, mode) for mode in (0, 1, 2)]
        np.testing.assert_allclose(got, ref[k], rtol=1e-14, atol=1e-17, err_msg=f"list {k}")


def test_chemical_potential_matches_reference(oracle_mod, case):
    elements, coeffs, n, species, g, lat, m = case
    alpha = S.alphabet(elements)
    solvent = alpha.index("Al")
    lat15 = oracle_mod.Lattice(15)
    m15 = oracle_mod.Model(elements, coeffs, lat15)
    pure = np.full(4 * 15 ** 3, solvent, np.int8)
    e_pure, _ = oracle_mod.energy(m15, lat15, pure)
    mu = []
    for c in range(len(alpha)):
        one = pure.copy()
        one[0] = c
        mu.append(0.0 if c == solvent else oracle_mod.energy(m15, lat15, one)[0] - e_pure)
    np.testing.assert_allclose(mu, g["mu"], rtol=1e-12, atol=1e-15)


def _bfs_clusters(lat, sp, solvent, smallest, bond):
    nb = [lat.neighbors(i)[:12] for i in range(sp.size)]
    seen = np.zeros(sp.size, bool)
    out = []
    for s0 in range(sp.size):
        if sp[s0] == solvent or seen[s0]:
            continue
        comp, q = [], deque([s0])
        seen[s0] = True
        while q:
            a = q.popleft()
            comp.append(a)
            for b in nb[a]:
                if sp[b] != solvent and not seen[b]:
                    seen[b] = True
                    q.append(int(b))
        if len(comp) < smallest:
            continue
        members = set(comp)
        if len(comp) > bond:
            shell = {int(b) for a in comp for b in nb[a]} - members
            for c in shell:
                if sum(1 for d in nb[c] if int(d) in members and sp[d] != solvent) > bond:
                    members.add(c)
        out.append(sorted(members))
    out.sort(key=lambda c: (-len(c), c[0]))
    return out


@pytest.mark.parametrize("smallest,bond", [(1, 12), (2, 3), (3, 2), (1, 0)])
def test_cluster_search_matches_breadth_first(oracle_mod, smallest, bond):
    el = ("Al", "Mg", "Zn")
    sp = S.make_lattice(8, {"Al": 0.78, "Mg": 0.12, "Zn": 0.10}, 2, 91, el)
    lat = oracle_mod.Lattice(8)
    got = oracle_mod.solute_clusters(lat, sp, 0, smallest, bond)
    want = _bfs_clusters(lat, sp, 0, smallest, bond)
    assert [c.tolist() for c in got] == want
    assert len(got) > 3


def test_site_de_matches_reference(oracle_mod):
    """GetDeFromAtomIdSite (EnergyChangePredictorPairSite.cpp:148-192), the building block of
    ExitTime's binding and profile energies, against the reference's own values
    (tests/golden/site_de_quaternary.npz): 310 (site, from, to) queries on the case lattice with its
    vacancies filled by the solvent."""
    from tests.golden.make_golden import site_de_lattice
    elements, coeffs, n, sp, vac = site_de_lattice()
    g = np.load("tests/golden/site_de_quaternary.npz")
    lat = oracle_mod.Lattice(n)
    m = oracle_mod.Model(elements, coeffs, lat)
    got = []
    for site, f, t in g["queries"]:
        x = sp.copy()
        x[site] = f
        got.append(oracle_mod.site_de(m, lat, x, int(site), int(t)))
    np.testing.assert_array_equal(np.asarray(got), g["de"])


def test_cluster_energy_over_every_site_is_the_census(oracle_mod, case):
    """GetEncodeOfCluster restricted to the whole lattice enumerates exactly GetEncode's clusters: the
    cluster energy of the list of every site equals the census energy, bit for bit."""
    elements, coeffs, n, species, g, lat, m = case
    solvent = S.alphabet(elements).index("Al")
    e_census, _ = oracle_mod.energy(m, lat, species)
    assert oracle_mod.cluster_energy(m, lat, species, solvent, np.arange(species.size), 0) == e_census


def test_cluster_info_fields(oracle_mod):
    """api.cluster_info: the mass-free fields of GetClustersInfo for the oracle's clusters; positions
    from the closed-form ids equal the oracle's restated GenerateFCC + ReassignLatticeVector
    positions, and a cluster straddling the periodic boundary gets its centre across the boundary."""
    from latticemontecarlo_gb300 import api
    el = ("Al", "Mg", "Zn")
    alpha = S.alphabet(el)
    n = 8
    sp = S.make_lattice(n, {"Al": 0.8, "Mg": 0.1, "Zn": 0.1}, 1, 5, el)
    lat = oracle_mod.Lattice(n)
    ids = np.arange(sp.size)
    np.testing.assert_allclose(api.site_relative_positions(n, ids), [lat.position(int(i)) for i in ids], atol=1e-15)
    clusters = oracle_mod.solute_clusters(lat, sp, alpha.index("Al"), 2, 3)
    ef = np.linspace(-0.1, 0.1, len(clusters))
    info = api.cluster_info(clusters, ef, sp, n, alpha)
    for k, (c, d) in enumerate(zip(clusters, info)):
        counts = np.bincount(sp[c], minlength=len(alpha))
        assert d["cluster_id"] == k + 1 and d["elements_number"]["Mg"] == counts[alpha.index("Mg")]
        assert d["cluster_size"] == len(c) - counts[alpha.index("X")]
        np.testing.assert_allclose(d["effective_radius"], (3 * len(c) * 4.046 ** 3 / 4 / (4 * np.pi)) ** (1 / 3))
        np.testing.assert_allclose(d["cluster_energy"], ef[k] / d["cluster_size"])
    # two neighbouring sites across the x boundary: the centre sits at the boundary, not mid-box
    a = 0                                   # h = (0, 0, 0)
    b = (2 * n - 1) * 2 * n * n + n * 0 + 0  # h = (2n - 1, 0, 1): a 1NN of site 0 across x
    (d,) = api.cluster_info([np.array([a, b])], [0.0], np.array([1] * (4 * n ** 3), np.int8), n, alpha)
    assert d["geometry_center"][0] > 0.9 * n * 4.046 or d["geometry_center"][0] < 0.1 * n * 4.046


def _ref_circular(rel, w):
    """GetGeometryCenter / GetMassCenter (SoluteCluster.cpp:412-455), restated with loops."""
    out = []
    for dim in range(3):
        sc = ss = sw = 0.0
        for r, m in zip(rel, w):
            sc += np.cos(r[dim] * 2 * np.pi) * m
            ss += np.sin(r[dim] * 2 * np.pi) * m
            sw += m
        out.append((np.arctan2(-ss / sw, -sc / sw) + np.pi) / (2 * np.pi))
    return np.array(out)


def _ref_wrap(v):
    while v >= 0.5:
        v -= 1
    while v < -0.5:
        v += 1
    return v


def test_cluster_info_geometry_and_mass_fields(oracle_mod):
    """Every field of GetClustersInfo against a loop-for-loop restatement of the reference's
    formulas on the oracle's positions (GenerateFCC + ReassignLatticeVector restated): the geometry
    and mass centres in all three coordinates, the full elements_number dict (X included), the mass,
    the gyration tensor and its eigenvalue measures (SelfAdjointEigenSolver's ascending order),
    the inertia tensor, and the frame-level aggregates (SoluteCluster.cpp:254-275)."""
    from latticemontecarlo_gb300 import api
    el = ("Al", "Cu", "Mg", "Zn")
    alpha = S.alphabet(el)
    mass = {"X": 0.0, "Al": 26.98, "Mg": 24.31, "Zn": 65.38, "Cu": 63.55}  # Element.hpp:71-87
    n = 8
    sp = S.make_lattice(n, {"Al": 0.8, "Cu": 0.05, "Mg": 0.08, "Zn": 0.07}, 3, 8, el)
    lat = oracle_mod.Lattice(n)
    clusters = oracle_mod.solute_clusters(lat, sp, alpha.index("Al"), 1, 3)
    ef = np.linspace(-0.2, 0.2, len(clusters))
    frame = api.clusters_frame_info(clusters, ef, sp, n, alpha)
    box = n * 4.046
    for c, d in zip(clusters, frame["clusters"]):
        rel = np.array([lat.position(int(i)) for i in c])
        w = np.array([mass[alpha[sp[i]]] for i in c])
        assert d["elements_number"] == {a: int(np.count_nonzero(sp[c] == k)) for k, a in enumerate(alpha)}
        assert np.array_equal(d["cluster_atom_id_list"], c)
        np.testing.assert_allclose(d["geometry_center"], _ref_circular(rel, np.ones(len(c))) * box, atol=1e-12)
        np.testing.assert_allclose(d["cluster_mass"], w.sum(), rtol=1e-15)
        if w.sum() == 0:
            continue  # a cluster of vacancies has no mass centre (0 / 0 in the reference too)
        mc = _ref_circular(rel, w)
        np.testing.assert_allclose(d["mass_center"], mc * box, atol=1e-12)
        gyr = np.zeros((3, 3))
        inertia = np.zeros((3, 3))
        for r, m in zip(rel, w):
            dr = np.array([_ref_wrap(r[k] - mc[k]) for k in range(3)])
            gyr += np.outer(dr, dr) * m
            cd = dr * box
            inertia += m * (np.dot(cd, cd) * np.eye(3) - np.outer(cd, cd))
        gyr = gyr / w.sum() * box * box
        np.testing.assert_allclose(d["mass_gyration_tensor"], gyr, rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(d["mass_inertia_tensor"], inertia, rtol=1e-12, atol=1e-9)
        if len(c) > 1:
            l1, l2, l3 = np.linalg.eigvalsh(gyr)
            np.testing.assert_allclose(d["mass_gyration_radius"], np.sqrt(l1 + l2 + l3), rtol=1e-12)
            np.testing.assert_allclose(d["asphericity"], l3 - 0.5 * (l1 + l2), atol=1e-10)
            np.testing.assert_allclose(d["acylindricity"], l2 - l1, atol=1e-10)
            np.testing.assert_allclose(d["anisotropy"], 1.5 * (l1 ** 2 + l2 ** 2 + l3 ** 2) / (l1 + l2 + l3) ** 2 - 0.5,
                                       atol=1e-10)
        else:
            assert np.isnan(d["mass_gyration_radius"])
    sizes = [len(c) - int(np.count_nonzero(sp[c] == alpha.index("X"))) for c in clusters]
    assert frame["num_cluster"] == len(clusters) and frame["num_atom"] == sum(sizes)
    assert frame["cluster_size_list"] == [str(v) for v in sizes]
    for k, a in enumerate(alpha):
        if a != "X":
            assert frame["num_" + a] == sum(int(np.count_nonzero(sp[c] == k)) for c in clusters)
    assert "num_X" not in frame
