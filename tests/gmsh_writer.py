"""gmsh 2.2 ASCII writer of periodic box meshes (QUAD in 2D, HEX in 3D), for the gmsh reader's tests.

The node grid has (n+1) points per direction; every node on a high side is the periodic image of the node on the low
side ($Periodic: one entity per direction, slave -> master node pairs; corners chain through two or three
entities).  Options exercise the reader: per-element vertex rotations (the element's first vertex at another corner),
mirrored (clockwise) vertex order, shuffled node numbering, boundary elements with periodic physical tags, a missing
$Periodic section (non-periodic boundaries), and an extra triangle.
"""
import numpy as np


def _grid_index(ijk, n):
    d = len(n)
    idx, stride = 0, 1
    for a in range(d):
        idx += ijk[a] * stride
        stride *= n[a] + 1
    return idx


def write_box_msh(path, d, n, lo, hi, rotate_seed=None, mirror_every=0, shuffle_seed=None, boundary_elements=True,
                  periodic=True, add_triangle=False, side_tags=None, periodic_dirs=None):
    """side_tags: {(direction, side): physical tag} of the boundary elements (default 10051 + 2 direction + side,
    the reference's PERIODIC_XL .. ZR on straight boundaries); periodic_dirs: the directions written to $Periodic
    (default all)."""
    n = tuple(n[:d])
    shape = tuple(k + 1 for k in n)
    n_nodes = int(np.prod(shape))
    coords = np.zeros((n_nodes, 3))
    for flat in range(n_nodes):
        ijk, r = [], flat
        for a in range(d):
            ijk.append(r % shape[a])
            r //= shape[a]
        for a in range(d):
            coords[flat, a] = lo[a] + (hi[a] - lo[a]) * ijk[a] / n[a]
    number = np.arange(1, n_nodes + 1)
    if shuffle_seed is not None:
        number = np.random.default_rng(shuffle_seed).permutation(n_nodes) + 1
    rng = np.random.default_rng(rotate_seed) if rotate_seed is not None else None

    elements = []   # (type, tags, node numbers)
    cells = [tuple(c) for c in np.ndindex(*tuple(reversed(n)))]
    for c_rev in cells:
        c = tuple(reversed(c_rev))
        tp = []
        for kv in range(1 << d):
            ijk = [c[a] + ((kv >> a) & 1) for a in range(d)]
            tp.append(_grid_index(ijk, n))
        if d == 2:
            ring = [tp[0], tp[1], tp[3], tp[2]]                  # counter-clockwise
            r = int(rng.integers(4)) if rng is not None else 0
            ring = ring[r:] + ring[:r]
            if mirror_every and len(elements) % mirror_every == 0:
                ring = ring[::-1]
            elements.append((3, (9401, 4001), ring))
        else:
            bot, top = [tp[0], tp[1], tp[3], tp[2]], [tp[4], tp[5], tp[7], tp[6]]
            r = int(rng.integers(4)) if rng is not None else 0
            bot, top = bot[r:] + bot[:r], top[r:] + top[:r]
            if mirror_every and len(elements) % mirror_every == 0:
                bot, top = bot[::-1], top[::-1]
            elements.append((5, (9401, 4001), bot + top))
    if boundary_elements:   # the periodic boundaries' lines / quadrilaterals (read past by the volume-based reader)
        for a in range(d):
            for side in (0, 1):
                tag = (side_tags or {}).get((a, side), 10051 + 2 * a + side)
                others = [b for b in range(d) if b != a]
                for c in np.ndindex(*[n[b] for b in others]):
                    pts = []
                    for kv in range(1 << (d - 1)):
                        ijk = [0] * d
                        ijk[a] = side * n[a]
                        for t, b in enumerate(others):
                            ijk[b] = c[t] + ((kv >> t) & 1)
                        pts.append(_grid_index(ijk, n))
                    if d == 2:
                        elements.append((1, (tag, 1000 + a), pts))
                    else:
                        elements.append((3, (tag, 1000 + a), [pts[0], pts[1], pts[3], pts[2]]))
    if add_triangle:
        elements.append((2, (9401, 4001), [0, 1, shape[0]]))

    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % n_nodes)
        order = np.argsort(number)
        for i in order:
            x = coords[i]
            f.write("%d %.17g %.17g %.17g\n" % (number[i], x[0], x[1], x[2]))
        f.write("$EndNodes\n$Elements\n%d\n" % len(elements))
        for k, (typ, tags, nodes) in enumerate(elements):
            f.write("%d %d %d %s %s\n" % (k + 1, typ, len(tags), " ".join(map(str, tags)),
                                          " ".join(str(number[q]) for q in nodes)))
        f.write("$EndElements\n")
        if periodic:
            dirs = list(range(d)) if periodic_dirs is None else list(periodic_dirs)
            f.write("$Periodic\n%d\n" % len(dirs))
            for a in dirs:
                pairs = []
                for flat in range(n_nodes):
                    ijk, r = [], flat
                    for b in range(d):
                        ijk.append(r % shape[b])
                        r //= shape[b]
                    if ijk[a] == n[a]:
                        m = list(ijk)
                        m[a] = 0
                        pairs.append((number[flat], number[_grid_index(m, n)]))
                f.write("%d %d %d\n%d\n" % (d - 1, 10052 + 2 * a, 10051 + 2 * a, len(pairs)))
                for s, m in pairs:
                    f.write("%d %d\n" % (s, m))
            f.write("$EndPeriodic\n")


def write_tri_msh(path, n, lo, hi, rotate_seed=None, flip_every=0, shuffle_seed=None, jitter=0.0, jitter_seed=0):
    """gmsh 2.2 periodic mesh of n[0] x n[1] cells each split into two triangles along the diagonal (i,j)-(i+1,j+1),
    with $Periodic correspondences in x and y.  Options: rotations of each triangle's vertex list, clockwise
    (flipped) triangles, shuffled node numbers, and periodic-consistent vertex jitter (uniform in +-jitter h)."""
    nx, ny = n
    shape = (nx + 1, ny + 1)
    n_nodes = shape[0] * shape[1]
    rng_j = np.random.default_rng(jitter_seed)
    jit = rng_j.uniform(-1.0, 1.0, size=(nx, ny, 2)) * jitter * np.array([(hi[0] - lo[0]) / nx, (hi[1] - lo[1]) / ny])
    coords = np.zeros((n_nodes, 3))
    for j in range(shape[1]):
        for i in range(shape[0]):
            q = i + shape[0] * j
            coords[q, 0] = lo[0] + (hi[0] - lo[0]) * i / nx + jit[i % nx, j % ny, 0]
            coords[q, 1] = lo[1] + (hi[1] - lo[1]) * j / ny + jit[i % nx, j % ny, 1]
    number = np.arange(1, n_nodes + 1)
    if shuffle_seed is not None:
        number = np.random.default_rng(shuffle_seed).permutation(n_nodes) + 1
    rng = np.random.default_rng(rotate_seed) if rotate_seed is not None else None
    node = lambda i, j: i + shape[0] * j
    elements = []
    for j in range(ny):
        for i in range(nx):
            for tri in ([node(i, j), node(i + 1, j), node(i + 1, j + 1)], [node(i, j), node(i + 1, j + 1), node(i, j + 1)]):
                if rng is not None:
                    r = int(rng.integers(3))
                    tri = tri[r:] + tri[:r]
                if flip_every and len(elements) % flip_every == 0:
                    tri = tri[::-1]
                elements.append((2, (9401, 4001), tri))
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % n_nodes)
        for q in np.argsort(number):
            x = coords[q]
            f.write("%d %.17g %.17g %.17g\n" % (number[q], x[0], x[1], x[2]))
        f.write("$EndNodes\n$Elements\n%d\n" % len(elements))
        for k, (typ, tags, nodes) in enumerate(elements):
            f.write("%d %d %d %s %s\n" % (k + 1, typ, len(tags), " ".join(map(str, tags)),
                                          " ".join(str(number[q]) for q in nodes)))
        f.write("$EndElements\n$Periodic\n2\n")
        for a in range(2):
            pairs = []
            for j in range(shape[1]):
                for i in range(shape[0]):
                    if (i == nx if a == 0 else j == ny):
                        m = (0, j) if a == 0 else (i, 0)
                        pairs.append((number[node(i, j)], number[node(*m)]))
            f.write("1 %d %d\n%d\n" % (10052 + 2 * a, 10051 + 2 * a, len(pairs)))
            for s_, m_ in pairs:
                f.write("%d %d\n" % (s_, m_))
        f.write("$EndPeriodic\n")


def write_tet_msh(path, n, lo, hi, rotate_seed=None, shuffle_seed=None):
    """gmsh 2.2 periodic mesh of n[0] x n[1] x n[2] cells each split into six tetrahedra along the diagonal
    (0,0,0)-(1,1,1) of the cell (for each axis permutation pi: (0,0,0), e_pi0, e_pi0 + e_pi1, (1,1,1)), with $Periodic
    correspondences in x, y and z.  Options: even permutations of each tetrahedron's vertex list (orientation kept)
    or, every third element, an odd one (negatively oriented in the file), and shuffled node numbers."""
    nx, ny, nz = n
    shape = (nx + 1, ny + 1, nz + 1)
    node = lambda i, j, k: i + shape[0] * (j + shape[1] * k)
    n_nodes = shape[0] * shape[1] * shape[2]
    coords = np.zeros((n_nodes, 3))
    for k in range(shape[2]):
        for j in range(shape[1]):
            for i in range(shape[0]):
                coords[node(i, j, k)] = [lo[0] + (hi[0] - lo[0]) * i / nx, lo[1] + (hi[1] - lo[1]) * j / ny,
                                         lo[2] + (hi[2] - lo[2]) * k / nz]
    number = np.arange(1, n_nodes + 1)
    if shuffle_seed is not None:
        number = np.random.default_rng(shuffle_seed).permutation(n_nodes) + 1
    rng = np.random.default_rng(rotate_seed) if rotate_seed is not None else None
    even = [(0, 1, 2, 3), (1, 2, 0, 3), (2, 0, 1, 3), (0, 2, 3, 1), (1, 3, 2, 0), (3, 1, 0, 2)]
    elements = []
    for k in range(nz):
        for j in range(ny):
            for i in range(nx):
                for pm in ((0, 1, 2), (0, 2, 1), (1, 0, 2), (1, 2, 0), (2, 0, 1), (2, 1, 0)):
                    c = [[0, 0, 0], [0, 0, 0], [0, 0, 0], [1, 1, 1]]
                    c[1][pm[0]] = 1
                    c[2][pm[0]] = 1
                    c[2][pm[1]] = 1
                    tet = [node(i + a, j + b, k + cc) for a, b, cc in c]
                    if rng is not None:
                        tet = [tet[q] for q in even[int(rng.integers(len(even)))]]
                    if len(elements) % 3 == 0:
                        tet = [tet[1], tet[0], tet[2], tet[3]]
                    elements.append((4, (9401, 4001), tet))
    with open(path, "w") as f:
        f.write("$MeshFormat\n2.2 0 8\n$EndMeshFormat\n$Nodes\n%d\n" % n_nodes)
        for q in np.argsort(number):
            x = coords[q]
            f.write("%d %.17g %.17g %.17g\n" % (number[q], x[0], x[1], x[2]))
        f.write("$EndNodes\n$Elements\n%d\n" % len(elements))
        for e, (typ, tags, nodes) in enumerate(elements):
            f.write("%d %d %d %s %s\n" % (e + 1, typ, len(tags), " ".join(map(str, tags)),
                                          " ".join(str(number[q]) for q in nodes)))
        f.write("$EndElements\n$Periodic\n3\n")
        for a in range(3):
            pairs = []
            for k in range(shape[2]):
                for j in range(shape[1]):
                    for i in range(shape[0]):
                        g = [i, j, k]
                        if g[a] == n[a]:
                            m = list(g)
                            m[a] = 0
                            pairs.append((number[node(*g)], number[node(*m)]))
            f.write("2 %d %d\n%d\n" % (10052 + 2 * a, 10051 + 2 * a, len(pairs)))
            for s_, m_ in pairs:
                f.write("%d %d\n" % (s_, m_))
        f.write("$EndPeriodic\n")
