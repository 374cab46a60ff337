"""Seeded synthetic bcc Fe / H systems for the saddle-search inner loop.

Every builder returns plain numpy arrays in the reference's layout: positions (N, 3) float64
(interleaved xyz per atom, system/adaptor.hpp:77), types (N,) uint32 (0 = Fe, 1 = H, the order of
the bundled wen.eam.fs table), frozen (N,) uint8, plus box extents and periodicity (orthorhombic).
"""
from __future__ import annotations

import os
from dataclasses import dataclass, field

import numpy as np

FE, H = 0, 1
A_FE = 2.855  # lattice parameter used by apps/hydrogen.cpp:114-116

TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "wen.eam.fs")

# Tetrahedral interstitial sites of the bcc conventional cell (fractions of a): four on each of
# the three faces through the cell origin.
TETRA = np.array(
    [[0.5, 0.25, 0.0], [0.5, 0.75, 0.0], [0.25, 0.5, 0.0], [0.75, 0.5, 0.0],
     [0.0, 0.5, 0.25], [0.0, 0.5, 0.75], [0.0, 0.25, 0.5], [0.0, 0.75, 0.5],
     [0.5, 0.0, 0.25], [0.5, 0.0, 0.75], [0.25, 0.0, 0.5], [0.75, 0.0, 0.5]])


@dataclass
class System:
    pos: np.ndarray          # (N, 3) float64
    types: np.ndarray        # (N,) uint32
    frozen: np.ndarray       # (N,) uint8
    extents: np.ndarray      # (3,) float64
    periodic: np.ndarray     # (3,) int32
    meta: dict = field(default_factory=dict)

    @property
    def n(self) -> int:
        return int(self.pos.shape[0])


def bcc_sites(nx: int, ny: int, nz: int, a: float) -> np.ndarray:
    """Sites of an nx*ny*nz bcc supercell in template_for order (x fastest, core.hpp:452-506),
    corner site then body centre in each cell."""
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cells = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1).astype(np.float64)
    out = np.empty((cells.shape[0] * 2, 3), dtype=np.float64)
    out[0::2] = cells * a
    out[1::2] = (cells + 0.5) * a
    return out


def kat_lattice(erase: bool = True) -> System:
    """The reference's EAM known-answer cell (tests/potential/EAM/eam.cpp:36-96): 7x7x7 bcc Fe at the
    300 K lattice parameter, fully periodic, site 1 erased when ``erase``."""
    T = 300.0
    V = 11.64012 + T * (9.37798e-5 + T * (3.643134e-7 + T * (1.851593e-10 + T * 5.669148e-14)))
    a = (2 * V) ** (1.0 / 3)
    sites = bcc_sites(7, 7, 7, a)
    if erase:
        sites = np.delete(sites, 1, axis=0)
    n = sites.shape[0]
    return System(sites, np.zeros(n, np.uint32), np.zeros(n, np.uint8), np.full(3, 7 * a), np.ones(3, np.int32),
                  dict(a=a))


def fe_vacancy_cell(seed: int = 1334) -> System:
    """6x6x6 bcc Fe (432 sites, a = 2.855), one vacancy at the central site, seeded Gaussian noise
    sigma = 0.02 A, periodic. meta['centre'] is the vacancy's nearest neighbour the search centres on."""
    rng = np.random.default_rng(seed)
    sites = bcc_sites(6, 6, 6, A_FE)
    L = 6 * A_FE
    centre_site = np.argmin(np.linalg.norm(sites - L / 2, axis=1))
    vac = sites[centre_site].copy()
    sites = np.delete(sites, centre_site, axis=0)
    d = np.linalg.norm(sites - vac, axis=1)
    nn = int(np.argmin(d))
    pos = sites + rng.normal(0.0, 0.02, sites.shape)
    n = pos.shape[0]
    return System(pos, np.zeros(n, np.uint32), np.zeros(n, np.uint8), np.full(3, L), np.ones(3, np.int32),
                  dict(centre=nn, vacancy=vac))


def perturb(sys: System, centre: int, rng: np.random.Generator, stddev: float = 0.6, r_pert: float = 4.0):
    """Master::perturb (find.cpp:1147-1214) with numpy's generator: sigma ~ N(stddev, stddev/3)
    truncated > 0; neighbours within r_pert of ``centre`` (minimum image) get Gaussian noise with the
    linear envelope (1 - r/r_pert) and Gaussian axis components; the centre gets full noise. Returns
    (positions, unit axis)."""
    s = -1.0
    while s < 0:
        s = rng.normal(stddev, stddev / 3.0)
    pos = sys.pos.copy()
    axis = np.zeros_like(pos)
    d = pos - pos[centre]
    L = sys.extents
    per = sys.periodic.astype(bool)
    d[:, per] -= L[per] * np.round(d[:, per] / L[per])
    r = np.linalg.norm(d, axis=1)
    sel = (r < r_pert) & (np.arange(sys.n) != centre) & (sys.frozen == 0)
    k = int(sel.sum())
    pos[sel] += rng.normal(0.0, s, (k, 3)) * (1.0 - r[sel] / r_pert)[:, None]
    axis[sel] += rng.normal(0.0, 1.0, (k, 3))
    pos[centre] += rng.normal(0.0, s, 3)
    axis[centre] += rng.normal(0.0, 1.0, 3)
    axis /= np.linalg.norm(axis)
    return pos, axis


def fe_h_crystal(n_cells: int = 80, seed: int = 2024) -> System:
    """n_cells^3 bcc Fe (80^3 = 1,024,000 sites): 0.1 % of sites vacated at random, H equal to 0.05 %
    of the atom count on random distinct tetrahedral sites, seeded sigma = 0.05 A displacements,
    periodic. Atoms are returned in site order with the H appended."""
    rng = np.random.default_rng(seed)
    sites = bcc_sites(n_cells, n_cells, n_cells, A_FE)
    n_sites = sites.shape[0]
    n_vac = int(round(0.001 * n_sites))
    keep = np.ones(n_sites, dtype=bool)
    keep[rng.choice(n_sites, n_vac, replace=False)] = False
    fe = sites[keep]
    n_h = int(round(0.0005 * fe.shape[0]))
    n_tet = n_cells ** 3 * TETRA.shape[0]
    pick = rng.choice(n_tet, n_h, replace=False)
    cell = pick // TETRA.shape[0]
    cz, rem = np.divmod(cell, n_cells * n_cells)
    cy, cx = np.divmod(rem, n_cells)
    h = (np.stack([cx, cy, cz], axis=1) + TETRA[pick % TETRA.shape[0]]) * A_FE
    pos = np.concatenate([fe, h]) + rng.normal(0.0, 0.05, (fe.shape[0] + n_h, 3))
    types = np.concatenate([np.zeros(fe.shape[0], np.uint32), np.ones(n_h, np.uint32)])
    n = pos.shape[0]
    return System(pos, types, np.zeros(n, np.uint8), np.full(3, n_cells * A_FE), np.ones(3, np.int32),
                  dict(n_vac=n_vac, n_h=n_h))


@dataclass
class Cluster:
    sys: System
    axis: np.ndarray     # (N, 3) unit dimer axis (zero on frozen atoms)
    centre: int


def cluster(rng: np.random.Generator, radius: float, shell: float = 5.5, n_vac: int = 0, n_h: int = 0,
            sigma_lattice: float = 0.02, sigma_centre: float = 0.1, margin: float = 3.0) -> Cluster:
    """A spherical cluster of ``radius`` cut around a lattice site of a perturbed bcc Fe lattice. Atoms
    further than radius - shell from the centre are frozen. ``n_vac`` first-/second-shell sites of the
    centre are vacated and ``n_h`` H sit on tetrahedral sites near the centre. Mobile atoms get
    sigma_centre displacements and the dimer axis is a random unit vector over them. The box is
    non-periodic and encloses the cluster with ``margin`` on every side."""
    m = int(np.ceil(radius / A_FE)) + 1
    g = np.arange(-m, m + 1, dtype=np.float64)
    k, j, i = np.meshgrid(g, g, g, indexing="ij")
    cells = np.stack([i.ravel(), j.ravel(), k.ravel()], axis=1)
    sites = np.concatenate([cells * A_FE, (cells + 0.5) * A_FE])
    d = np.linalg.norm(sites, axis=1)
    sites = sites[d <= radius]
    d = d[d <= radius]
    order = np.argsort(d, kind="stable")
    sites, d = sites[order], d[order]
    if n_vac:
        near = np.nonzero((d > 0.1) & (d < 3.0))[0]
        drop = rng.choice(near, min(n_vac, near.size), replace=False)
        keep = np.ones(sites.shape[0], dtype=bool)
        keep[drop] = False
        sites, d = sites[keep], d[keep]
    types = np.zeros(sites.shape[0], np.uint32)
    if n_h:
        tet = (cells[:, None, :] + TETRA[None, :, :]).reshape(-1, 3) * A_FE
        td = np.linalg.norm(tet, axis=1)
        cand = np.nonzero((td > 1.0) & (td < 3.2))[0]
        hs = tet[rng.choice(cand, min(n_h, cand.size), replace=False)]
        sites = np.concatenate([sites, hs])
        d = np.concatenate([d, np.linalg.norm(hs, axis=1)])
        types = np.concatenate([types, np.ones(hs.shape[0], np.uint32)])
    pos = sites + rng.normal(0.0, sigma_lattice, sites.shape)
    frozen = (d > radius - shell).astype(np.uint8)
    active = frozen == 0
    if not active.any():  # keep at least the centre mobile
        frozen[int(np.argmin(d))] = 0
        active = frozen == 0
    pos[active] += rng.normal(0.0, sigma_centre, (int(active.sum()), 3))
    axis = np.zeros_like(pos)
    axis[active] = rng.normal(0.0, 1.0, (int(active.sum()), 3))
    axis /= np.linalg.norm(axis)
    lo = pos.min(axis=0) - margin
    pos = pos - lo
    ext = pos.max(axis=0) + margin
    centre = int(np.argmin(d))
    s = System(pos, types, frozen, ext, np.zeros(3, np.int32),
               dict(radius=radius, n_vac=n_vac, n_h=int((types == H).sum())))
    return Cluster(s, axis, centre)


def served_box(seed: int = 16, cells: int = 20, n_vac: int = 5, n_h: int = 20) -> System:
    """The served workload's system: cells^3 bcc Fe (20^3 = 16,000 sites) with n_vac vacancies and n_h H
    on random distinct tetrahedral sites, seeded sigma = 0.02 A noise, periodic."""
    rng = np.random.default_rng(seed)
    sites = bcc_sites(cells, cells, cells, A_FE)
    keep = np.ones(sites.shape[0], dtype=bool)
    vac = rng.choice(sites.shape[0], n_vac, replace=False)
    keep[vac] = False
    pick = rng.choice(cells ** 3 * TETRA.shape[0], n_h, replace=False)
    cz, rem = np.divmod(pick // TETRA.shape[0], cells * cells)
    cy, cx = np.divmod(rem, cells)
    h = (np.stack([cx, cy, cz], axis=1) + TETRA[pick % TETRA.shape[0]]) * A_FE
    pos = np.concatenate([sites[keep], h])
    pos += rng.normal(0.0, 0.02, pos.shape)
    types = np.concatenate([np.zeros(int(keep.sum()), np.uint32), np.ones(n_h, np.uint32)])
    n = pos.shape[0]
    return System(pos, types, np.zeros(n, np.uint8), np.full(3, cells * A_FE), np.ones(3, np.int32),
                  dict(vacancies=sites[vac], n_fe=int(keep.sum())))


def environment_centres(box: System, n_env: int, rng: np.random.Generator) -> np.ndarray:
    """Atoms whose local environments a KMC step would emit searches for: the H atoms, the nearest
    neighbours of each vacancy, then random Fe atoms."""
    L = box.extents
    cand = list(np.nonzero(box.types == H)[0])
    for v in box.meta["vacancies"]:
        d = box.pos - v
        d -= L * np.round(d / L)
        cand += list(np.argsort(np.linalg.norm(d, axis=1))[:8])
    cand = list(dict.fromkeys(int(c) for c in cand))
    rng.shuffle(cand)
    while len(cand) < n_env:
        cand.append(int(rng.integers(0, box.meta["n_fe"])))
    return np.array(cand[:n_env])


def cut_request(box: System, centre: int, radius: float, rng: np.random.Generator, shell: float = 5.5,
                margin: float = 3.0, stddev: float = 0.6, r_pert: float = 4.0) -> Cluster:
    """One served search request: the atoms within ``radius`` of ``centre`` (minimum image) as a
    non-periodic cluster with a frozen outer shell, perturbed and given an axis as Master::perturb does
    (find.cpp:1147-1214: sigma ~ N(stddev, stddev/3) > 0, envelope 1 - r/r_pert on the mobile
    neighbours within r_pert, full noise on the centre)."""
    L = box.extents
    d = box.pos - box.pos[centre]
    d -= L * np.round(d / L)
    r = np.linalg.norm(d, axis=1)
    sel = np.nonzero(r <= radius)[0]
    sel = sel[np.argsort(r[sel], kind="stable")]
    pos = d[sel].copy()
    rr = r[sel]
    frozen = (rr > radius - shell).astype(np.uint8)
    frozen[0] = 0
    sub = System(pos, box.types[sel].copy(), frozen, np.ones(3), np.zeros(3, np.int32))
    s = -1.0
    while s < 0:
        s = rng.normal(stddev, stddev / 3.0)
    axis = np.zeros_like(pos)
    near = (rr < r_pert) & (frozen == 0)
    near[0] = False
    k = int(near.sum())
    pos[near] += rng.normal(0.0, s, (k, 3)) * (1.0 - rr[near] / r_pert)[:, None]
    axis[near] = rng.normal(0.0, 1.0, (k, 3))
    pos[0] += rng.normal(0.0, s, 3)
    axis[0] = rng.normal(0.0, 1.0, 3)
    axis /= np.linalg.norm(axis)
    lo = pos.min(axis=0) - margin
    pos -= lo
    sub.pos = pos
    sub.extents = pos.max(axis=0) + margin
    sub.meta = dict(radius=radius, box_index=sel)
    return Cluster(sub, axis, 0)


def served_requests(n_env: int = 96, seed: int = 44, r_min: float = 6.0, r_max: float = 11.0,
                    per_env: tuple[int, int] = (8, 32)):
    """The served request stream: n_env new local environments in the 16,000-site box, each emitting
    8-32 searches of clusters with radius ~ U(r_min, r_max). Returns a list of (environment, Cluster)."""
    rng = np.random.default_rng(seed)
    box = served_box()
    out = []
    for e, c in enumerate(environment_centres(box, n_env, rng)):
        for _ in range(int(rng.integers(per_env[0], per_env[1] + 1))):
            out.append((e, cut_request(box, int(c), rng.uniform(r_min, r_max), rng)))
    return out


def search_clusters(n: int = 4096, seed: int = 7, r_min: float = 6.0, r_max: float = 11.0) -> list[Cluster]:
    """n independent clusters with radii ~ U(r_min, r_max), 0-3 vacancies, 0-2 H (all seeded)."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        r = rng.uniform(r_min, r_max)
        out.append(cluster(rng, r, n_vac=int(rng.integers(0, 4)), n_h=int(rng.integers(0, 3))))
    return out
