"""Mesh, node types and initial state: the caller-side set-up of a run.

This is what the reference's g_init (props.F90:52-235) and ptcl_init
(ptcl_lib.F90:15-30) produce, for a single block (px = py = 1), plus the mesh
law and seeded initial state of the 2D argon DC glow workloads:

* ``mesh_law='uniform'`` and ``'tanh'`` follow props.F90:96-124 operation by
  operation, including its REAL(4) literals (2.0*1.175/float(nx+1)).
* ``mesh_law='geometric'``: node spacing grows by ``ratio`` per cell away
  from each electrode (x = 0 and x = l) until it reaches ``cap`` times the
  spacing at the electrode, then stays uniform; the spacings are scaled so
  the nodes span [0, l] exactly.  (A pure 1.05 progression over 512 cells per
  half-gap would span a factor 1.05**511 ~ 6e10 in spacing.)
* y is uniform as in the reference.

Arrays follow the reference layout: Fortran column-major (nx+2, ny+2), ghost
ring included, so ``ni[i-1, j-1]`` is Fortran ``ni(i, j)``.
"""
import numpy as np

F32 = np.float32


def _sp(v):
    """A REAL(4) literal promoted to REAL(8)."""
    return float(F32(v))


class Mesh:
    """Node coordinates, spacings and node types of one 2D grid."""

    def __init__(self, nx, ny, x, y, type_x, type_y):
        self.nx, self.ny = int(nx), int(ny)
        self.x = np.ascontiguousarray(x, dtype=np.float64)            # nx+2
        self.y = np.ascontiguousarray(y, dtype=np.float64)            # ny+2
        self.dx = np.ascontiguousarray(self.x[1:] - self.x[:-1])      # nx+1
        self.dlx = np.ascontiguousarray(0.5 * (self.dx[1:] + self.dx[:-1]))
        self.dy = np.ascontiguousarray(self.y[1:] - self.y[:-1])
        self.dly = np.ascontiguousarray(0.5 * (self.dy[1:] + self.dy[:-1]))
        self.r = self.y.copy()
        self.type_x = np.asfortranarray(type_x, dtype=np.int32)       # (nx, ny)
        self.type_y = np.asfortranarray(type_y, dtype=np.int32)

    def c_struct(self):
        """fs_mesh pointing into this object's arrays (keep self alive)."""
        from .abi import FsMesh, dptr, iptr
        self._tx_flat = np.ascontiguousarray(self.type_x.ravel(order="F"))
        self._ty_flat = np.ascontiguousarray(self.type_y.ravel(order="F"))
        return FsMesh(dptr(self.dx), dptr(self.dlx), dptr(self.dy), dptr(self.dly),
                      dptr(self.r), iptr(self._tx_flat), iptr(self._ty_flat))


def x_nodes(nx, l, law="geometric", ratio=1.05, cap=4.0):
    n = nx + 2
    if law == "uniform":
        x = np.array([l / float(F32(nx + 1)) * (i - 1) for i in range(1, n + 1)])
    elif law == "tanh":
        xt = float(F32(F32(2.0) * F32(1.175)) / F32(nx + 1))
        x = np.tanh(-_sp(1.175) + xt * np.arange(0, n, dtype=np.float64))
    elif law == "geometric":
        k = np.arange(nx + 1)
        d = np.minimum(k, nx - k).astype(np.float64)
        s = np.minimum(ratio ** d, cap)
        x = np.concatenate([[0.0], np.cumsum(s)])
    else:
        raise ValueError("unknown mesh law %r" % law)
    # props.F90:109-116: shift to 0, normalise by the last node, scale to l
    x = x - x[0]
    x = x / x[-1]
    x = x * l
    return x


def y_nodes(ny, w):
    """Uniform y nodes, props.F90:138-155."""
    y = np.array([w / float(F32(ny + 1)) * (j - 1) for j in range(1, ny + 3)])
    y = y - y[0]
    y = y / y[-1]
    y = y * w
    return y


def node_types(nx, ny, y, ew, gap, rwall=False):
    """type_x / type_y of props.F90:182-218 for one block."""
    tx = np.zeros((nx, ny), dtype=np.int32, order="F")
    ty = np.zeros((nx, ny), dtype=np.int32, order="F")
    for j in range(1, ny + 1):
        for i in range(1, nx + 1):
            if j == 1:
                ty[i - 1, j - 1] = -1
            if j == ny:
                ty[i - 1, j - 1] = 3 if rwall else 1
            yj = y[j - 1]
            elec = (yj <= ew) or (yj >= gap)
            if i == 1:
                tx[i - 1, j - 1] = -2 if elec else -1
            if i == nx:
                tx[i - 1, j - 1] = 2 if elec else 1
    return tx, ty


def make_mesh(nx, ny, l, w, ew, gap, law="geometric", ratio=1.05, cap=4.0, rwall=False):
    if nx < 3 or ny < 2:
        raise ValueError("nx >= 3 and ny >= 2 are required")
    x = x_nodes(nx, l, law, ratio, cap)
    y = y_nodes(ny, w)
    tx, ty = node_types(nx, ny, y, ew, gap, rwall)
    return Mesh(nx, ny, x, y, tx, ty)


# ------------------------------------------------------------ initial state
_M64 = (1 << 64) - 1


def splitmix64(z):
    """splitmix64 finaliser on a uint64 numpy array (vectorised)."""
    z = (z + np.uint64(0x9E3779B97F4A7C15)) & np.uint64(_M64)
    z = ((z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)) & np.uint64(_M64)
    z = ((z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)) & np.uint64(_M64)
    return z ^ (z >> np.uint64(31))


def uniform_pm1(seed, stream, n):
    """n deterministic samples of U(-1, 1) from splitmix64(seed, stream, index)."""
    with np.errstate(over="ignore"):
        base = np.uint64((seed * 0x100000001B3 + stream * 0x9E3779B1) & _M64)
        z = splitmix64(np.arange(n, dtype=np.uint64) + base * np.uint64(0x10001))
    u = (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return 2.0 * u - 1.0


def blob_state(mesh, consts, peak_m3=1e14, floor_m3=1e8, sigma_m=1e-3,
               energy_ev=1.0, noise=0.0, seed=0, vl=None):
    """Quasi-neutral Gaussian blob at the gap centre on a density floor.

    Returns Fortran-ordered (nx+2, ny+2) arrays ni, ne, nt (nt = ne * energy / ph0,
    i.e. mean energy ``energy_ev``) and ph.  With ``noise`` > 0 each
    species density is multiplied by (1 + noise*U(-1,1)), U from a
    counter-based generator seeded by (seed, species, cell index).

    ph is zero inside.  With ``vl`` (nondimensional applied voltage) its
    electrode ghost columns hold +vl/2 at x = 0 and -vl/2 at x = l, the values
    circ_step writes there (circ_lib.F90:185-194), so the applied voltage is on
    from t = 0.  Without it they are 0 as after ptcl_init/lapl_init, and the
    first RK stage then sees different boundary potentials than the next four.
    """
    x0 = consts["x0"]
    ph0 = consts["ph0"]
    X, Y = np.meshgrid(mesh.x, mesh.y, indexing="ij")
    xc, yc = mesh.x[-1] / 2.0, mesh.y[-1] / 2.0
    sig = sigma_m / x0
    r2 = (X - xc) ** 2 + (Y - yc) ** 2
    n = (floor_m3 + peak_m3 * np.exp(-r2 / (2.0 * sig * sig))) * x0 ** 3
    shape = n.shape
    ni = n.copy()
    ne = n.copy()
    if noise > 0:
        ni = ni * (1.0 + noise * uniform_pm1(seed, 0, n.size).reshape(shape, order="F"))
        ne = ne * (1.0 + noise * uniform_pm1(seed, 1, n.size).reshape(shape, order="F"))
    nt = ne * (energy_ev / ph0)
    ph = np.zeros(shape)
    if vl is not None:
        ph[0, :] = vl / 2.0
        ph[-1, :] = vl / (-2.0)
    f = np.asfortranarray
    return dict(ni=f(ni), ne=f(ne), nt=f(nt), ph=f(ph))
