"""Lattice geometry, unit cells and bond lists (host-side set-up).

The unit-cell table restates unit_cell.h:27-127; the point generators follow
the row/column rules of utilities.h (createPlateHEX2D :118-168,
createCuboidSC3D :170-211), anchored at the origin; the bond rule is
Assembly::createBonds (assembly.h:212-234): a directed bond i -> j for every
j != i with |x_i - x_j| < 1.01 * cutoff[1], layer 0 when it is also below
1.01 * cutoff[0].  Bonds come out ordered by (i, j), which is the order
createBonds pushes them into Particle::bond_layers.
"""
import math

import numpy as np

SQUARE2D, HEXAGON2D, SIMPLECUBIC3D, FCC3D, BCC3D = "Square2D", "Hexagon2D", "SimpleCubic3D", "FCC3D", "BCC3D"


class UnitCell:
    """Per-lattice constants of unit_cell.h (same names as the reference)."""

    # el_mapping data as written in unit_cell.h, row by row
    _TABLE = {
        SQUARE2D: dict(data=[1 / 2, -1 / 2, 0, 0, 0, 1 / 2, 0, 1 / 12, -1 / 12], dim=2, nneighbors=8,
                       nneighbors1=4, nneighbors2=4, cut=(2.0, 2.0 * math.sqrt(2.0)), afem=(16, 12, 12),
                       vol=lambda r: 4 * r ** 2),
        HEXAGON2D: dict(data=[math.sqrt(3.0) / 12.0, -math.sqrt(3.0) / 12.0, 0, -math.sqrt(3.0) / 144.0,
                              math.sqrt(3.0) / 48.0, 0, 0, 0, 1.0], dim=2, nneighbors=12, nneighbors1=6,
                        nneighbors2=6, cut=(2.0, 2.0 * math.sqrt(3.0)), afem=(30, 18, 18),
                        vol=lambda r: 2 * math.sqrt(3) * r ** 2),
        SIMPLECUBIC3D: dict(data=[1, -1, -1.0, 0, 0, 1.0, 0, 1 / 18.0, -1 / 18.0], dim=3, nneighbors=18,
                            nneighbors1=6, nneighbors2=12, cut=(2.0, 2.0 * math.sqrt(2.0)), afem=(60, 24, 54),
                            vol=lambda r: (2 * r) ** 3),
        FCC3D: dict(data=[0, 0, math.sqrt(2.0), math.sqrt(2.0) / 4, -math.sqrt(2.0) / 4, -math.sqrt(2.0) / 4, 0,
                          math.sqrt(2.0) / 24, -math.sqrt(2.0) / 24], dim=3, nneighbors=18, nneighbors1=12,
                    nneighbors2=6, cut=(2.0, 2.0 * math.sqrt(2.0)), afem=(60, 54, 24),
                    vol=lambda r: 4.0 * math.sqrt(2.0) * r ** 3),
        BCC3D: dict(data=[0, 0, math.sqrt(3.0), 1 / math.sqrt(3.0), -1 / math.sqrt(3.0), 0, 0, math.sqrt(3.0) / 14,
                          math.sqrt(3.0) / 14], dim=3, nneighbors=14, nneighbors1=8, nneighbors2=6,
                    cut=(2.0, 4.0 / math.sqrt(3.0)), afem=(40, 34, 24),
                    vol=lambda r: 32.0 * math.sqrt(3.0) / 9.0 * r ** 3),
    }

    def __init__(self, lattice, radius):
        t = self._TABLE[lattice]
        self.lattice = lattice
        self.radius = float(radius)
        self.dim = t["dim"]
        self.nneighbors = t["nneighbors"]
        self.nneighbors1 = t["nneighbors1"]
        self.nneighbors2 = t["nneighbors2"]
        self.nneighbors_AFEM, self.nneighbors_AFEM1, self.nneighbors_AFEM2 = t["afem"]
        self.neighbor_cutoff = [t["cut"][0] * radius, t["cut"][1] * radius]
        self.particle_volume = t["vol"](radius)
        self._data = np.array(t["data"], dtype=np.float64)

    def el_mapping(self, layout="reference"):
        """3x3 mapping from (C11, C12, C44) to (Kn, Tv) terms.

        ``reference``: the matrix the reference builds, Eigen::Map over the
        written data, which reads it column by column (unit_cell.h:49 etc.).
        ``row``: the written rows applied as rows, which gives the physical
        constants (Kn = r*C44, Tv = r*(C12-C44)/18 for the simple cubic cell).
        """
        m = self._data.reshape(3, 3)
        return m.T.copy() if layout == "reference" else m.copy()

    def elastic_constants(self, E=None, nu=None, plane_stress=False, C=None, layout="reference"):
        """(Kn, Tv) per layer as ParticleElastic::setParticleProperty computes
        them (particle_elastic.h:70-143): returns (Kn_layer0, Kn_layer1, Tv)."""
        if C is None:
            if not plane_stress:
                C11 = E * (1.0 - nu) / (1.0 + nu) / (1.0 - 2.0 * nu)
                C12 = E * nu / (1.0 + nu) / (1.0 - 2.0 * nu)
                C44 = E / 2.0 / (1.0 + nu)
            else:
                C11 = E / (1.0 - nu) / (1.0 + nu)
                C12 = E * nu / (1.0 + nu) / (1.0 - nu)
                C44 = E / 2.0 / (1.0 + nu)
            C = (C11, C12, C44)
        M = self.el_mapping(layout)
        Ce = np.asarray(C, dtype=np.float64)
        k = np.array([M[i, 0] * Ce[0] + M[i, 1] * Ce[1] + M[i, 2] * Ce[2] for i in range(3)])
        if self.dim == 3:
            k = self.radius * k
        if self.lattice == HEXAGON2D:
            return float(k[0]), float(k[0]), float(k[1])
        return float(k[0]), float(k[1]), float(k[2])


    def elastic_constants_grad(self, E, nu, plane_stress=False, layout="reference"):
        """Derivatives of elastic_constants(E, nu) = (Kn0, Kn1, Tv) with
        respect to E and nu: a (2, 3) array, rows d/dE and d/dnu."""
        if not plane_stress:
            D = (1.0 + nu) * (1.0 - 2.0 * nu)
            dC_dE = np.array([(1.0 - nu) / D, nu / D, 0.5 / (1.0 + nu)])
            dC_dnu = np.array([2.0 * E * nu * (2.0 - nu) / D ** 2, E * (1.0 + 2.0 * nu * nu) / D ** 2,
                               -0.5 * E / (1.0 + nu) ** 2])
        else:
            q = 1.0 - nu * nu
            dC_dE = np.array([1.0 / q, nu / q, 0.5 / (1.0 + nu)])
            dC_dnu = np.array([2.0 * E * nu / q ** 2, E * (1.0 + nu * nu) / q ** 2, -0.5 * E / (1.0 + nu) ** 2])
        out = np.zeros((2, 3))
        for r, dC in enumerate((dC_dE, dC_dnu)):
            out[r] = self.elastic_constants(C=tuple(dC), layout=layout)  # the map is linear in C
        return out


def hex_plate(ncol, nrow, a):
    """Hexagonal plate: even rows hold ncol points, odd rows ncol-1 points
    shifted by a/2 (the createPlateHEX2D row rule); row pitch a*sqrt(3)/2."""
    hy = a * math.sqrt(3.0) / 2.0
    pts = []
    for j in range(nrow):
        if j % 2 == 0:
            xs = a * np.arange(ncol, dtype=np.float64)
        else:
            xs = a * (2 * np.arange(ncol - 1, dtype=np.float64) + 1) / 2.0
        pts.append(np.stack([xs, np.full_like(xs, hy * j), np.zeros_like(xs)], axis=1))
    return np.concatenate(pts, axis=0)


def sc_cuboid(nx, ny, nz, a):
    """Simple cubic grid of nx*ny*nz points, x fastest (createCuboidSC3D order)."""
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    return np.stack([a * i.ravel(), a * j.ravel(), a * k.ravel()], axis=1).astype(np.float64)


def bcc_cuboid(nx, ny, nz, a):
    """BCC grid: corner points of an nx*ny*nz cell block plus body centres,
    ordered by z, then y, then x (corners and centres interleaved by layer)."""
    pts = []
    for kz in range(nz + 1):
        k, j, i = np.meshgrid([kz], np.arange(ny + 1), np.arange(nx + 1), indexing="ij")
        pts.append(np.stack([a * i.ravel(), a * j.ravel(), a * k.ravel()], axis=1))
        if kz < nz:
            k, j, i = np.meshgrid([kz], np.arange(ny), np.arange(nx), indexing="ij")
            pts.append(np.stack([a * (i.ravel() + 0.5), a * (j.ravel() + 0.5), a * (k.ravel() + 0.5)], axis=1))
    return np.concatenate(pts, axis=0).astype(np.float64)


def find_bonds(xyz, cell):
    """Directed bonds (p1, p2, layer) with the createBonds rule and order.

    Candidate pairs come from a k-d tree; each is then accepted with the
    reference's own arithmetic (sqrt of the summed squared differences,
    compared with 1.01 * cutoff), so the result matches the O(N^2) search.
    """
    from scipy.spatial import cKDTree

    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    c0 = 1.01 * cell.neighbor_cutoff[0]
    c1 = 1.01 * cell.neighbor_cutoff[1]
    tree = cKDTree(xyz)
    pairs = tree.query_pairs(c1 * (1 + 1e-9) + 1e-12, output_type="ndarray")
    i = np.concatenate([pairs[:, 0], pairs[:, 1]])
    j = np.concatenate([pairs[:, 1], pairs[:, 0]])
    d = xyz[i] - xyz[j]
    dist = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    keep = (dist < c1) & (i != j)
    i, j, dist = i[keep], j[keep], dist[keep]
    order = np.lexsort((j, i))
    i, j, dist = i[order], j[order], dist[order]
    layer = np.where(dist < c0, 0, 1).astype(np.int32)
    return i.astype(np.int32), j.astype(np.int32), layer


def bond_constants(cell, layer, KnTv):
    """Per-bond Kn, Tv from (Kn0, Kn1, Tv) (particle_elastic.h:112-124)."""
    kn0, kn1, tv = KnTv
    Kn = np.where(layer == 0, kn0, kn1).astype(np.float64)
    Tv = np.full(layer.shape, tv, dtype=np.float64)
    return Kn, Tv


def nonlocal_neighbors(xyz, cutoff):
    """Assembly::searchNonlocalNeighbors (assembly.h:117-130): for every
    particle, the ids (ascending, itself included) closer than `cutoff`
    (= cutoff_ratio * nonlocal_L), as CSR (ptr, idx)."""
    from scipy.spatial import cKDTree

    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    tree = cKDTree(xyz)
    pairs = tree.query_pairs(cutoff * (1 + 1e-9) + 1e-12, output_type="ndarray")
    n = len(xyz)
    i = np.concatenate([pairs[:, 0], pairs[:, 1], np.arange(n)])
    j = np.concatenate([pairs[:, 1], pairs[:, 0], np.arange(n)])
    d = xyz[i] - xyz[j]
    dist = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    keep = dist < cutoff
    i, j = i[keep], j[keep]
    order = np.lexsort((j, i))
    i, j = i[order], j[order]
    ptr = np.zeros(n + 1, np.int64)
    np.add.at(ptr, i + 1, 1)
    return np.cumsum(ptr), j.astype(np.int32)


def weibull_draws(p1, p2, shape, scale, seed):
    """One draw per undirected bond, shared by its two directed copies:
    scale * (-ln(1 - U))^(1/shape) with U uniform from a seeded generator,
    the pairs {i, j} taken in ascending (min, max) order."""
    p1 = np.asarray(p1, dtype=np.int64)
    p2 = np.asarray(p2, dtype=np.int64)
    n = int(max(p1.max(initial=0), p2.max(initial=0))) + 1
    key = np.minimum(p1, p2) * n + np.maximum(p1, p2)
    uniq, inv = np.unique(key, return_inverse=True)
    u = np.random.default_rng(seed).random(len(uniq))
    return (scale * (-np.log1p(-u)) ** (1.0 / shape))[inv]


def precrack(xyz, p1, p2, layer, y0, x_tip):
    """Deletes the bonds whose segment crosses the line y = y0 left of x_tip
    (a straight edge crack; geometry/geo1_CT_configuration.cpp:79-134 filters
    its bond list against a notch region the same way); both directed copies
    of a bond go together.  Returns the kept (p1, p2, layer)."""
    xyz = np.asarray(xyz, dtype=np.float64)
    y1, y2 = xyz[p1, 1], xyz[p2, 1]
    cross = (y1 - y0) * (y2 - y0) < 0
    t = np.where(cross, (y0 - y1) / np.where(cross, y2 - y1, 1.0), 0.0)
    xc = xyz[p1, 0] + t * (xyz[p2, 0] - xyz[p1, 0])
    keep = ~(cross & (xc < x_tip))
    return p1[keep], p2[keep], layer[keep]


def sent_plate(ncol, nrow, a, crack_ratio=0.3):
    """Single-edge-notched plate: hexagonal lattice (hex_plate rows) with a
    crack from the left edge along the mid-height line between two rows,
    of length crack_ratio * W.  Returns (xyz, p1, p2, layer, cell)."""
    cell = UnitCell(HEXAGON2D, a / 2)
    xyz = hex_plate(ncol, nrow, a)
    p1, p2, layer = find_bonds(xyz, cell)
    h = a * math.sqrt(3.0) / 2.0
    y0 = (nrow // 2 - 0.5) * h
    W = xyz[:, 0].max() - xyz[:, 0].min()
    p1, p2, layer = precrack(xyz, p1, p2, layer, y0, xyz[:, 0].min() + crack_ratio * W)
    return xyz, p1, p2, layer, cell


def random_rotations(n, rng):
    """n rotation matrices uniform on SO(3), from uniform unit quaternions
    (Shoemake's subgroup algorithm)."""
    u1, u2, u3 = rng.random(n), rng.random(n), rng.random(n)
    q = np.stack([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)], axis=1)
    x, y, z, w = q[:, 0], q[:, 1], q[:, 2], q[:, 3]
    R = np.empty((n, 3, 3))
    R[:, 0, 0] = 1 - 2 * (y * y + z * z)
    R[:, 0, 1] = 2 * (x * y - z * w)
    R[:, 0, 2] = 2 * (x * z + y * w)
    R[:, 1, 0] = 2 * (x * y + z * w)
    R[:, 1, 1] = 1 - 2 * (x * x + z * z)
    R[:, 1, 2] = 2 * (y * z - x * w)
    R[:, 2, 0] = 2 * (x * z - y * w)
    R[:, 2, 1] = 2 * (y * z + x * w)
    R[:, 2, 2] = 1 - 2 * (x * x + y * y)
    return R


def bcc_polycrystal(ncell, a, ngrain, seed, overlap=0.5):
    """Voronoi polycrystal of BCC grains in the cube [0, ncell*a]^3, built the
    way the reference's Fortran Mbuilder does (benchmark/BCC_Hailong/
    create_BCC_configuration.F90:169-333): for every grain, a BCC lattice of
    cubic cell a rotated by the grain's orientation about its seed, the sites
    inside the grain's Voronoi cell and the box kept, and sites closer than
    overlap * (nearest-neighbour distance) to an earlier grain's particle
    dropped.  Seeds are uniform in the box and orientations uniform on SO(3),
    from one seeded generator.  Returns (xyz, grain id per particle)."""
    from scipy.spatial import cKDTree

    rng = np.random.default_rng(seed)
    L = ncell * a
    seeds = rng.random((ngrain, 3)) * L
    R = random_rotations(ngrain, rng)
    # bounding box of each Voronoi cell inside the box, from a sampling grid
    m = 48
    g = (np.arange(m) + 0.5) / m * L
    G = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    owner = cKDTree(seeds).query(G)[1]
    pad = L / m
    parts, gid = [], []
    tree = None
    thr = overlap * a * math.sqrt(3.0) / 2.0
    for k in range(ngrain):
        P = G[owner == k]
        if len(P) == 0:
            continue
        lo, hi = P.min(0) - pad, P.max(0) + pad
        corners = np.array([[x, y, z] for x in (lo[0], hi[0]) for y in (lo[1], hi[1]) for z in (lo[2], hi[2])])
        local = (corners - seeds[k]) @ R[k]  # grain frame: x_local = R^T (x - seed)
        i0 = np.floor(local.min(0) / a).astype(int) - 1
        i1 = np.ceil(local.max(0) / a).astype(int) + 1
        ax = [np.arange(i0[d], i1[d] + 1) for d in range(3)]
        C = np.stack(np.meshgrid(*ax, indexing="ij"), -1).reshape(-1, 3).astype(np.float64) * a
        sites = np.concatenate([C, C + 0.5 * a])
        X = sites @ R[k].T + seeds[k]
        inbox = np.all((X >= 0.0) & (X <= L), axis=1)
        X = X[inbox]
        X = X[cKDTree(seeds).query(X)[1] == k]
        if tree is not None and len(X):
            near = tree.query(X, distance_upper_bound=thr)[0]
            X = X[~np.isfinite(near) | (near >= thr)]
        parts.append(X)
        gid.append(np.full(len(X), k, np.int32))
        tree = cKDTree(np.concatenate(parts))
    return np.concatenate(parts), np.concatenate(gid)


def prune_weak(xyz, cell, min_bonds):
    """Indices of the particles kept after repeatedly dropping those with
    fewer than min_bonds bonds (createBonds rule).  Grain-boundary and
    surface particles of a polycrystal can end up with two or three bonds,
    too few to hold them in 3-D: their stiffness has a null direction and
    the Newton system becomes singular."""
    keep = np.arange(len(xyz))
    while True:
        p1, _, _ = find_bonds(xyz[keep], cell)
        nb = np.bincount(p1, minlength=len(keep))
        ok = nb >= min_bonds
        if ok.all():
            return keep
        keep = keep[ok]


def _in_notch(x, y, tip, half_width):
    """The wedge notch of geometry/geo1_CT_configuration.cpp:54-64: within
    half_width of the notch line and inside the 30-degree wedge that opens
    from the tip towards +x."""
    dy = y - tip[1]
    return (np.abs(dy) <= half_width) & (dy >= (tip[0] - x) / math.sqrt(3.0)) & (dy <= (x - tip[0]) / math.sqrt(3.0))


def ct_specimen(W, a0_ratio, a, notch_half_width=None):
    """Compact-tension plate on a hexagonal lattice of spacing a, ASTM E647
    proportions in the layout of the reference's CT builder
    (geometry/geo1_CT_configuration.cpp:120-160): back edge at x = 0, load
    line at x = W, plate 1.25 W wide and 1.2 W high, pin holes of diameter
    0.25 W centred on the load line at 0.275 W above and below the crack
    line y = 0.6 W, and a wedge notch from the right edge to the tip at
    x = W - a0_ratio*W.  Particles inside the holes or the notch are dropped,
    and so is every bond that passes through them (tested at ten points
    along the bond, as the builder does).  Returns
    (xyz, p1, p2, layer, cell, info) with the hole centres, radius and tip."""
    cell = UnitCell(HEXAGON2D, a / 2)
    Lx, Ly = 1.25 * W, 1.2 * W
    ncol = int(math.floor(Lx / a)) + 1
    nrow = int(math.floor(Ly / (a * math.sqrt(3.0) / 2.0))) + 1
    xyz = hex_plate(ncol, nrow, a)
    yc, r = 0.6 * W, 0.125 * W
    holes = [(W, yc - 0.275 * W), (W, yc + 0.275 * W)]
    tip = (W - a0_ratio * W, yc)
    hw = notch_half_width if notch_half_width is not None else 0.026 * W

    def invalid(x, y):
        bad = _in_notch(x, y, tip, hw)
        for cx, cy in holes:
            bad |= (x - cx) ** 2 + (y - cy) ** 2 <= r * r
        return bad

    xyz = xyz[~invalid(xyz[:, 0], xyz[:, 1])]
    p1, p2, layer = find_bonds(xyz, cell)
    keep = np.ones(len(p1), dtype=bool)
    for k in range(10):
        t = (k + 0.5) / 10.0
        mx = xyz[p1, 0] + t * (xyz[p2, 0] - xyz[p1, 0])
        my = xyz[p1, 1] + t * (xyz[p2, 1] - xyz[p1, 1])
        keep &= ~invalid(mx, my)
    info = dict(holes=holes, radius=r, tip=tip, crack_y=yc, W=W)
    return xyz, p1[keep], p2[keep], layer[keep], cell, info


def ct_groups(xyz, info, a):
    """Load groups of LoadCTForce (load_step_fatigue.h:69-84): the particles
    on the upper face of the top hole and the lower face of the bottom hole
    within 30 degrees of the load line (pin contact), and the back-edge
    particles on the crack line (held in y)."""
    (cx, cy_b), (_, cy_t) = info["holes"]
    r = info["radius"]
    d_t = np.hypot(xyz[:, 0] - cx, xyz[:, 1] - cy_t)
    d_b = np.hypot(xyz[:, 0] - cx, xyz[:, 1] - cy_b)
    ring = 1.5 * a
    top = np.where((d_t < r + ring) & (xyz[:, 1] - cy_t > np.cos(np.pi / 6) * d_t))[0]
    bottom = np.where((d_b < r + ring) & (cy_b - xyz[:, 1] > np.cos(np.pi / 6) * d_b))[0]
    mid = np.where((xyz[:, 0] < 0.6 * a) & (np.abs(xyz[:, 1] - info["crack_y"]) < a))[0]
    return dict(top=top, bottom=bottom, mid=mid)
