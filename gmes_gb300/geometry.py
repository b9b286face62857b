"""Cartesian Yee grid and geometric primitives.

Interface mirror of the reference's ``gmes.geometry`` (gmes/geometry.py) and
of the Cython geometry module ``gmes.pygeom`` (src/pygeom.pyx).  The scalar
methods keep the reference's signatures and arithmetic; every shape also
has a vectorised ``contains(x, y, z)`` so that ``FDTD.init()`` can assign
materials to all Yee points with array operations instead of the
reference's per-point Python loop (gmes/fdtd.py:353-477).
"""

from copy import deepcopy
from math import sqrt

import numpy as np

from . import constant as const

# Yee staggering of each component in units of the cell size: the space
# coordinate of index n along an axis is (n + offset) * dr - half_size
# (gmes/geometry.py:360-732).  Rows are Ex, Ey, Ez, Hx, Hy, Hz.
YEE_OFFSET = np.array([
    [0.5, 0.0, 0.0],
    [0.0, 0.5, 0.0],
    [0.0, 0.0, 0.5],
    [0.0, -0.5, -0.5],
    [-0.5, 0.0, -0.5],
    [-0.5, -0.5, 0.0],
])


class AuxiCartComm:
    """Single-rank cyclic stand-in for an MPI Cartesian communicator.

    Same behaviour as gmes/geometry.py:16-101: ``Shift`` on a periodic axis
    returns (0, 0), so the ghost-plane exchange degenerates to a periodic
    copy inside the one domain.
    """

    def __init__(self, dims=(1, 1, 1), periods=None, reorder=(0, 0, 0)):
        self.rank = 0
        self.dim = 3
        cyclic = tuple(map(int, periods)) if periods else (0, 0, 0)
        self.topo = ((1, 1, 1), cyclic, (0, 0, 0))

    def Get_cart_rank(self, coords):
        return 0

    def Get_coords(self, rank):
        return 0, 0, 0

    def Get_dim(self):
        return self.dim

    def Get_topo(self):
        return self.topo

    def Get_size(self):
        return 1

    def Shift(self, direction, disp):
        return (0, 0) if self.topo[1][direction] else (-1, -1)

    def sendrecv(self, sendbuf, dest=0, sendtag=0, recvbuf=None, source=0,
                 recvtag=0, status=None):
        return None if dest == -1 or source == -1 else sendbuf

    def reduce(self, value, root=0, op=None):
        return value

    def bcast(self, obj=None, root=0):
        return obj

    def allgather(self, obj=None):
        return [obj]


class Cartesian:
    """The computational domain (gmes/geometry.py:104-358).

    ``whole_field_size`` = N; the component arrays have the staggered shapes
    Ex (Nx, Ny+1, Nz+1), Ey (Nx+1, Ny, Nz+1), Ez (Nx+1, Ny+1, Nz),
    Hx (Nx, Ny+1, Nz+1), Hy (Nx+1, Ny, Nz+1), Hz (Nx+1, Ny+1, Nz); an
    inactive component is (1, 1, 1).  The engine runs one domain on one GPU:
    ``parallel=True`` is accepted and ignored, as the reference does when
    mpi4py is absent.
    """

    def __init__(self, size, resolution=15, parallel=False):
        try:
            if len(resolution) == 3:
                self.res = np.array(resolution, np.double)
        except TypeError:
            self.res = np.array((resolution,) * 3, np.double)
        self.dr = np.array(1 / self.res, np.double)
        self.half_size = 0.5 * np.array(size, np.double)
        for i, v in enumerate(self.dr):
            if self.half_size[i] == 0:
                self.half_size[i] = 0.5 * v
        self.whole_field_size = np.array((2 * self.half_size * self.res).round(), np.intp)
        self.my_id = 0
        self.numprocs = 1
        self.cart_comm = AuxiCartComm((1, 1, 1), (1, 1, 1))
        self.my_cart_idx = self.cart_comm.Get_topo()[2]
        self.general_field_size = self.whole_field_size // self.cart_comm.Get_topo()[0]
        self.my_field_size = np.array(self.whole_field_size, np.intp)
        self.dt = None

    # -- storage -----------------------------------------------------------
    def field_shape(self, comp, field_compnt):
        """Array shape of ``comp`` when the active set is ``field_compnt``."""
        if comp not in field_compnt:
            return (1, 1, 1)
        n = [int(v) for v in self.my_field_size]
        c = comp.index
        shape = [n[0] + 1, n[1] + 1, n[2] + 1]
        own = c % 3
        shape[own] = n[own]
        return tuple(shape)

    def _storage(self, comp, field_compnt, cmplx):
        return np.zeros(self.field_shape(comp, field_compnt),
                        complex if cmplx else np.double)

    def get_ex_storage(self, field_compnt, cmplx=False):
        return self._storage(const.Ex, field_compnt, cmplx)

    def get_ey_storage(self, field_compnt, cmplx=False):
        return self._storage(const.Ey, field_compnt, cmplx)

    def get_ez_storage(self, field_compnt, cmplx=False):
        return self._storage(const.Ez, field_compnt, cmplx)

    def get_hx_storage(self, field_compnt, cmplx=False):
        return self._storage(const.Hx, field_compnt, cmplx)

    def get_hy_storage(self, field_compnt, cmplx=False):
        return self._storage(const.Hy, field_compnt, cmplx)

    def get_hz_storage(self, field_compnt, cmplx=False):
        return self._storage(const.Hz, field_compnt, cmplx)

    # -- index <-> space ---------------------------------------------------
    def axis_coords(self, comp, axis, n):
        """Space coordinates of indices 0..n-1 of ``comp`` along ``axis``.

        Same arithmetic as the scalar ``*_index_to_space`` methods
        (gmes/geometry.py:360-732): (idx + 0.5) * dr - half for a +1/2
        offset, (idx - 0.5) * dr - half for -1/2, idx * dr - half otherwise.
        """
        idx = np.arange(n, dtype=np.intp)
        off = YEE_OFFSET[comp.index][axis]
        if off == 0:
            return idx * self.dr[axis] - self.half_size[axis]
        return (idx + off) * self.dr[axis] - self.half_size[axis]

    def _index_to_space(self, comp, i, j, k):
        out = []
        for axis, n in enumerate((i, j, k)):
            off = YEE_OFFSET[comp.index][axis]
            g = int(n)
            if off == 0:
                out.append(g * self.dr[axis] - self.half_size[axis])
            else:
                out.append((g + off) * self.dr[axis] - self.half_size[axis])
        return tuple(np.float64(v) for v in out)

    def _space_to_exact(self, comp, x, y, z):
        coords = np.array((x, y, z), np.double)
        off = YEE_OFFSET[comp.index]
        g = np.empty(3, np.double)
        for a in range(3):
            g[a] = (coords[a] + self.half_size[a]) / self.dr[a] - off[a]
        if comp.index < 3:
            for a in range(3):
                if self.whole_field_size[a] == 1:
                    g[a] = 0
        else:
            own = comp.index % 3
            for a in range(3):
                if self.whole_field_size[a] == 1:
                    g[a] = 0 if a == own else 1
        return tuple(g)

    def _space_to_index(self, comp, x, y, z):
        exact = self._space_to_exact(comp, x, y, z)
        return tuple(np.floor(np.array(exact) + 0.5).astype(np.intp))

    def ex_index_to_space(self, i, j, k):
        return self._index_to_space(const.Ex, i, j, k)

    def ey_index_to_space(self, i, j, k):
        return self._index_to_space(const.Ey, i, j, k)

    def ez_index_to_space(self, i, j, k):
        return self._index_to_space(const.Ez, i, j, k)

    def hx_index_to_space(self, i, j, k):
        return self._index_to_space(const.Hx, i, j, k)

    def hy_index_to_space(self, i, j, k):
        return self._index_to_space(const.Hy, i, j, k)

    def hz_index_to_space(self, i, j, k):
        return self._index_to_space(const.Hz, i, j, k)

    def spc_to_exact_ex_idx(self, x, y, z):
        return self._space_to_exact(const.Ex, x, y, z)

    def spc_to_exact_ey_idx(self, x, y, z):
        return self._space_to_exact(const.Ey, x, y, z)

    def spc_to_exact_ez_idx(self, x, y, z):
        return self._space_to_exact(const.Ez, x, y, z)

    def spc_to_exact_hx_idx(self, x, y, z):
        return self._space_to_exact(const.Hx, x, y, z)

    def spc_to_exact_hy_idx(self, x, y, z):
        return self._space_to_exact(const.Hy, x, y, z)

    def spc_to_exact_hz_idx(self, x, y, z):
        return self._space_to_exact(const.Hz, x, y, z)

    def space_to_ex_index(self, x, y, z):
        return self._space_to_index(const.Ex, x, y, z)

    def space_to_ey_index(self, x, y, z):
        return self._space_to_index(const.Ey, x, y, z)

    def space_to_ez_index(self, x, y, z):
        return self._space_to_index(const.Ez, x, y, z)

    def space_to_hx_index(self, x, y, z):
        return self._space_to_index(const.Hx, x, y, z)

    def space_to_hy_index(self, x, y, z):
        return self._space_to_index(const.Hy, x, y, z)

    def space_to_hz_index(self, x, y, z):
        return self._space_to_index(const.Hz, x, y, z)

    def space_to_index(self, comp, x, y, z):
        return self._space_to_index(comp, x, y, z)

    def index_to_space(self, comp, i, j, k):
        return self._index_to_space(comp, i, j, k)

    def display_info(self, indent=0):
        print(" " * indent, "Cartesian space")
        print(" " * indent, "size:", 2 * self.half_size, "resolution:", self.res)
        print(" " * indent, "dx:", self.dr[0], "dy:", self.dr[1], "dz:", self.dr[2])


def in_range(idx, shape, component):
    """Whether ``idx`` is an updatable (non-ghost) point (gmes/geometry.py:751-812)."""
    c = component.index
    own = c % 3
    for a in range(3):
        if c < 3:
            hi = shape[a] if a == own else shape[a] - 1
            if idx[a] < 0 or idx[a] >= hi:
                return False
        else:
            lo_excl = a != own
            if (idx[a] <= 0 if lo_excl else idx[a] < 0) or idx[a] >= shape[a]:
                return False
    return True


# ---------------------------------------------------------------------------
# Geometric primitives (src/pygeom.pyx:477-1148)
# ---------------------------------------------------------------------------

def _norm(p):
    return sqrt(p[0] ** 2 + p[1] ** 2 + p[2] ** 2)


class GeomBox:
    """Axis-aligned bounding box (src/pygeom.pyx:160-250); bounds inclusive."""

    def __init__(self, low=(0, 0, 0), high=(0, 0, 0)):
        self.low = np.array(low, np.double)
        self.high = np.array(high, np.double)

    def union(self, box):
        self.low = np.minimum(self.low, box.low)
        self.high = np.maximum(self.high, box.high)

    def add_point(self, point):
        self.low = np.minimum(self.low, point)
        self.high = np.maximum(self.high, point)

    def in_box(self, point):
        return all(self.low[i] <= point[i] <= self.high[i] for i in range(3))

    def __str__(self):
        return "low: " + str(self.low) + " high: " + str(self.high)


class GeometricObject:
    """Base class of the shapes; ``material`` fills the shape."""

    def __init__(self, material):
        self.material = material
        self.box = None

    def init(self, space):
        self.material.init(space)
        self.box = self.geom_box()

    def geom_box(self):
        raise NotImplementedError

    def in_object(self, point):
        """Scalar inclusion test (same arithmetic as the reference)."""
        x, y, z = (np.array([v], np.double) for v in point)
        return bool(self.contains(x, y, z)[0])

    def contains(self, x, y, z):
        """Vectorised inclusion test over broadcastable coordinate arrays."""
        raise NotImplementedError

    def shape_record(self):
        """Fields of this shape's ``gmes_shape`` for the GPU rasteriser."""
        raise NotImplementedError

    def _record(self, kind, **kw):
        rec = {"type": kind, "compound": int(getattr(self.material, "compound", False)),
               "lo": [float(v) for v in self.box.low], "hi": [float(v) for v in self.box.high]}
        rec.update(kw)
        return rec

    def display_info(self, indent=0):
        if self.material:
            self.material.display_info(indent + 5)


class DefaultMedium(GeometricObject):
    """Fills the whole space (src/pygeom.pyx:538-568)."""

    def geom_box(self):
        return GeomBox((-np.inf,) * 3, (np.inf,) * 3)

    def contains(self, x, y, z):
        return np.ones(np.broadcast_shapes(np.shape(x), np.shape(y), np.shape(z)), bool)

    def shape_record(self):
        return self._record(0)


class Cone(GeometricObject):
    """Cone or truncated cone (src/pygeom.pyx:571-690)."""

    def __init__(self, material, center=(0, 0, 0), radius2=0, axis=(1, 0, 0),
                 radius=1, height=1):
        super().__init__(material)
        if radius < 0:
            raise ValueError("radius must be non-negative.")
        if radius2 < 0:
            raise ValueError("radius2 must be non-negative.")
        self.radius = float(radius)
        self.radius2 = float(radius2)
        self.center = np.array(center, np.double)
        self.axis = np.array(axis, np.double) / _norm(axis)
        self.height = float(height)

    def contains(self, x, y, z):
        rx, ry, rz = x - self.center[0], y - self.center[1], z - self.center[2]
        ax = self.axis
        proj = ax[0] * rx + ax[1] * ry + ax[2] * rz
        inside = np.abs(proj) <= 0.5 * self.height
        if self.radius2 == self.radius == np.inf:
            return inside
        radius = self.radius + (proj / self.height + 0.5) * (self.radius2 - self.radius)
        px, py, pz = rx - proj * ax[0], ry - proj * ax[1], rz - proj * ax[2]
        dist = np.sqrt(px ** 2 + py ** 2 + pz ** 2)
        return inside & (dist <= np.abs(radius))

    def shape_record(self):
        return self._record(4, center=list(self.center), axis=list(self.axis),
                            p=[self.radius, self.radius2, self.height])

    def geom_box(self):
        h = 0.5 * self.height
        radial = np.sqrt(np.maximum(0, 1 - self.axis * self.axis))
        e1 = np.zeros(3)
        e2 = np.zeros(3)
        np.multiply(self.radius, radial, out=e1, where=radial != 0)
        np.multiply(self.radius2, radial, out=e2, where=radial != 0)
        b1 = GeomBox(self.center - h * self.axis - e1, self.center - h * self.axis + e1)
        b2 = GeomBox(self.center + h * self.axis - e2, self.center + h * self.axis + e2)
        b1.union(b2)
        return b1


class Cylinder(Cone):
    """Right circular cylinder (src/pygeom.pyx:693-740)."""

    def __init__(self, material, center=(0, 0, 0), axis=(0, 0, 1), radius=1, height=1):
        super().__init__(material, center, radius, axis, radius, height)


class Block(GeometricObject):
    """Parallelepiped with edge directions e1, e2, e3 (src/pygeom.pyx:743-843)."""

    def __init__(self, material, center=(0, 0, 0), e1=(1, 0, 0), e2=(0, 1, 0),
                 e3=(0, 0, 1), size=(1, 1, 1)):
        super().__init__(material)
        self.center = np.array(center, np.double)
        self.e1 = np.array(e1, np.double) / _norm(e1)
        self.e2 = np.array(e2, np.double) / _norm(e2)
        self.e3 = np.array(e3, np.double) / _norm(e3)
        self.size = np.array(size, np.double)
        self.projection_matrix = np.linalg.inv(np.column_stack((self.e1, self.e2, self.e3)))

    def _proj(self, x, y, z):
        r = (x - self.center[0], y - self.center[1], z - self.center[2])
        m = self.projection_matrix
        return [m[a, 0] * r[0] + m[a, 1] * r[1] + m[a, 2] * r[2] for a in range(3)]

    def contains(self, x, y, z):
        p = self._proj(x, y, z)
        h = 0.5 * self.size
        return (np.abs(p[0]) <= h[0]) & (np.abs(p[1]) <= h[1]) & (np.abs(p[2]) <= h[2])

    def shape_record(self):
        return self._record(2, center=list(self.center),
                            m=[float(v) for v in self.projection_matrix.ravel()],
                            p=[float(v) for v in 0.5 * self.size])

    def geom_box(self):
        s1, s2, s3 = self.size[0] * self.e1, self.size[1] * self.e2, self.size[2] * self.e3
        corner = self.center - 0.5 * (s1 + s2 + s3)
        box = GeomBox(self.center, self.center)
        for c in (corner, corner + s1, corner + s2, corner + s3, corner + s1 + s2,
                  corner + s1 + s3, corner + s3 + s2, corner + s1 + s2 + s3):
            box.add_point(c)
        return box


class Ellipsoid(Block):
    """Ellipsoid inscribed in a Block (src/pygeom.pyx:846-894)."""

    def __init__(self, material, center=(0, 0, 0), e1=(1, 0, 0), e2=(0, 1, 0),
                 e3=(0, 0, 1), size=(1, 1, 1)):
        super().__init__(material, center, e1, e2, e3, size)
        self.inverse_semi_axes = 2 / np.array(size, np.double)

    def contains(self, x, y, z):
        p = self._proj(x, y, z)
        q = [p[a] * self.inverse_semi_axes[a] for a in range(3)]
        return (q[0] * q[0] + q[1] * q[1]) + q[2] * q[2] <= 1

    def shape_record(self):
        return self._record(3, center=list(self.center),
                            m=[float(v) for v in self.projection_matrix.ravel()],
                            p=[float(v) for v in self.inverse_semi_axes])


class Sphere(GeometricObject):
    """Sphere (src/pygeom.pyx:897-973): |p - center| <= radius."""

    def __init__(self, material, center=(0, 0, 0), radius=1):
        super().__init__(material)
        if radius < 0:
            raise ValueError("radius must be non-negative.")
        self.radius = float(radius)
        self.center = np.array(center, np.double)

    def contains(self, x, y, z):
        rx, ry, rz = x - self.center[0], y - self.center[1], z - self.center[2]
        return np.sqrt(rx ** 2 + ry ** 2 + rz ** 2) <= self.radius

    def geom_box(self):
        return GeomBox(self.center - self.radius, self.center + self.radius)

    def shape_record(self):
        return self._record(1, center=list(self.center), p=[self.radius, 0.0, 0.0])


class Shell(GeometricObject):
    """A slab shell of thickness ``thickness`` inside a box (src/pygeom.pyx:976-1148).

    Without ``size`` it lines the whole domain; this is how the absorbing
    boundaries (Cpml, Upml) are placed.
    """

    def __init__(self, material, center=(0, 0, 0), size=None, thickness=1,
                 plus_x=True, minus_x=True, plus_y=True, minus_y=True,
                 plus_z=True, minus_z=True):
        super().__init__(material)
        self.center = np.array(center, np.double)
        self.d = float(thickness)
        self.box_list = []
        self.minus_x, self.plus_x = minus_x, plus_x
        self.minus_y, self.plus_y = minus_y, plus_y
        self.minus_z, self.plus_z = minus_z, plus_z
        if size is None:
            self.half_size = np.zeros(3)
            self.boundary = True
        else:
            self.half_size = np.array([0.5 * v for v in size], np.double)
            self.boundary = False

    def init(self, space):
        if self.boundary:
            self.half_size = np.array(space.half_size, np.double)
        for i in range(3):
            if 2 * self.half_size[i] < space.dr[i]:
                self.half_size[i] = 0.5 * space.dr[i]
        flags = [[self.minus_x, self.plus_x], [self.minus_y, self.plus_y],
                 [self.minus_z, self.plus_z]]
        for i in range(3):
            if 2 * self.half_size[i] <= space.dr[i]:
                flags[i] = [False, False]
        (self.minus_x, self.plus_x), (self.minus_y, self.plus_y), \
            (self.minus_z, self.plus_z) = flags
        c, h, d = self.center, self.half_size, self.d
        self.box_list = []
        for axis, (minus, plus) in ((0, flags[0]), (1, flags[1]), (2, flags[2])):
            if plus:
                low = c - h
                low[axis] = c[axis] + h[axis] - d
                self.box_list.append(GeomBox(low, c + h))
            if minus:
                high = c + h
                high[axis] = c[axis] - h[axis] + d
                self.box_list.append(GeomBox(c - h, high))
        # the reference orders the slabs +x, -x, +y, -y, +z, -z; order does
        # not change the union
        self.material.init(space, (self.center, self.half_size, self.d))
        self.box = self.geom_box()

    def contains(self, x, y, z):
        shape = np.broadcast_shapes(np.shape(x), np.shape(y), np.shape(z))
        out = np.zeros(shape, bool)
        for b in self.box_list:
            out |= ((b.low[0] <= x) & (x <= b.high[0]) & (b.low[1] <= y) & (y <= b.high[1])
                    & (b.low[2] <= z) & (z <= b.high[2]))
        return out

    def geom_box(self):
        return GeomBox(self.center - self.half_size, self.center + self.half_size)

    def shape_record(self):
        return self._record(5, nbox=len(self.box_list),
                            box_lo=[[float(v) for v in b.low] for b in self.box_list],
                            box_hi=[[float(v) for v in b.high] for b in self.box_list])


class GeomBoxTree:
    """Point -> (material, underneath material) lookup.

    The reference builds a bounding-box tree (src/pygeom.pyx:300-474) whose
    answer is: the LAST object of the geometry list that contains the point,
    falling back to the first object (``find_object``,
    src/pygeom.pyx:143-156); for a ``Compound`` material (the PMLs) the
    "underneath" object is the last earlier object containing the point.
    The tree only accelerates that scan; this class answers the same
    question directly, and ``FDTD.init`` answers it for whole grids at once
    (``rasterize``).
    """

    def __init__(self, geom_list):
        self.geom_list = tuple(geom_list)

    def _find(self, point, upto):
        for i in range(upto - 1, 0, -1):
            if self.geom_list[i].in_object(point):
                return self.geom_list[i], i
        return self.geom_list[0], 0

    def object_of_point(self, point):
        obj, idx = self._find(tuple(point), len(self.geom_list))
        under = None
        if getattr(obj.material, "compound", False):
            under, _ = self._find(tuple(point), idx)
        return obj, under

    def material_of_point(self, point):
        obj, under = self.object_of_point(point)
        return obj.material, (under.material if under is not None else None)

    def display_info(self, indent=0):
        for g in self.geom_list:
            print(" " * indent, "bounding box:", g.box)
            g.display_info(indent + 5)


def rasterize(geom_list, coords):
    """Owner and underneath object index of every point of a Yee grid.

    ``coords`` = (xs, ys, zs), the 1-D coordinate arrays of one component.
    Returns int16 arrays (owner, under) of shape (len(xs), len(ys), len(zs)):
    ``owner`` is the index of the last object containing the point (0 when
    none of objects 1.. does), ``under`` the same search restricted to the
    objects before a Compound owner (-1 where the owner is not Compound).
    """
    xs, ys, zs = coords
    shape = (len(xs), len(ys), len(zs))
    owner = np.zeros(shape, np.int16)
    under = np.full(shape, -1, np.int16)
    X = xs[:, None, None]
    Y = ys[None, :, None]
    Z = zs[None, None, :]
    for m in range(1, len(geom_list)):
        g = geom_list[m]
        box = g.box
        # restrict the test to the points inside the (inclusive) bounding box
        sl = []
        for arr, lo, hi in ((xs, box.low[0], box.high[0]), (ys, box.low[1], box.high[1]),
                            (zs, box.low[2], box.high[2])):
            idx = np.nonzero((arr >= lo) & (arr <= hi))[0]
            if len(idx) == 0:
                sl = None
                break
            sl.append(slice(idx[0], idx[-1] + 1))
        if sl is None:
            continue
        sub = g.contains(X[sl[0]], Y[:, sl[1]], Z[:, :, sl[2]])
        sub = np.broadcast_to(sub, owner[tuple(sl)].shape)
        if not sub.any():
            continue
        region = owner[tuple(sl)]
        if getattr(g.material, "compound", False):
            uregion = under[tuple(sl)]
            uregion[sub] = region[sub]
        else:
            uregion = under[tuple(sl)]
            uregion[sub] = -1
        region[sub] = m
    return owner, under


__all__ = [
    "AuxiCartComm", "Cartesian", "in_range", "GeomBox", "GeomBoxTree",
    "GeometricObject", "DefaultMedium", "Cone", "Cylinder", "Block",
    "Ellipsoid", "Sphere", "Shell", "rasterize", "YEE_OFFSET",
]
