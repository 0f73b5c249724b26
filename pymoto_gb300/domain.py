"""Structured voxel domain with pyMOTO's numbering (pymoto/common/domain.py:58-428).

Only the numbering and geometry used by the hot path are provided.  The GPU modules accept either this
class or pyMOTO's own VoxelDomain (they read nelx/nely/nelz and unitx/unity/unitz only).
"""
import numpy as np


class VoxelDomain:
    """element (i,j,k) -> (k*nely + j)*nelx + i; node (i,j,k) -> (k*(nely+1) + j)*(nelx+1) + i."""

    def __init__(self, nelx: int, nely: int, nelz: int = 0, unitx: float = 1.0, unity: float = 1.0,
                 unitz: float = 1.0):
        self.nelx, self.nely, self.nelz = int(nelx), int(nely), int(nelz or 0)
        self.dim = 2 if self.nelz == 0 else 3
        self.origin = np.array([0.0, 0.0, 0.0])
        self.unitx, self.unity, self.unitz = float(unitx), float(unity), float(unitz)
        if np.prod(self.element_size[: self.dim]) <= 0:
            raise ValueError("Element volume needs to be positive")
        self.nel = self.nelx * self.nely * max(self.nelz, 1)
        self.nnodes = (self.nelx + 1) * (self.nely + 1) * (self.nelz + 1)
        self.elemnodes = 2 ** self.dim
        # local node a of an element sits at the corner with signs (x, y, z) = (+-1, +-1, +-1): bit 0 of a is x,
        # bit 1 is y, bit 2 is z (pyMOTO's local order, domain.py:132-142)
        self.node_numbering = [[1 if (a >> c) & 1 else -1 for c in range(3)] for a in range(self.elemnodes)]
        I, J, K = np.meshgrid(np.arange(self.nelx), np.arange(self.nely), np.arange(max(self.nelz, 1)),
                              indexing="ij")
        self.elements = self.get_elemnumber(I, J, K)
        I, J, K = np.meshgrid(np.arange(self.nelx + 1), np.arange(self.nely + 1), np.arange(self.nelz + 1),
                              indexing="ij")
        self.nodes = self.get_nodenumber(I, J, K)

    @property
    def element_size(self):
        return np.array([self.unitx, self.unity, self.unitz])

    @property
    def size(self):
        return np.array([self.nelx, self.nely, self.nelz])[: self.dim]

    @property
    def domain_size(self):
        return np.array([self.nelx * self.unitx, self.nely * self.unity, self.nelz * self.unitz])[: self.dim]

    def get_node_indices(self, nod_idx=None):
        """(i, j[, k]) of node number(s), stacked on the first axis (all nodes by default)."""
        n = np.arange(self.nnodes) if nod_idx is None else np.asarray(nod_idx)
        nx1, ny1 = self.nelx + 1, self.nely + 1
        ijk = [n % nx1, (n // nx1) % ny1] + ([n // (nx1 * ny1)] if self.dim == 3 else [])
        return np.stack(ijk, axis=0)

    def get_node_position(self, nod_idx=None):
        """Coordinates (dim, #nodes) of node number(s): origin + index * element size."""
        ijk = self.get_node_indices(nod_idx)
        return (self.origin[: self.dim] + self.element_size[: self.dim] * ijk.T).T

    def get_element_indices(self, el_idx=None):
        """(i, j[, k]) of element number(s), stacked on the first axis (all elements by default)."""
        e = np.arange(self.nel) if el_idx is None else np.asarray(el_idx)
        ijk = [e % self.nelx, (e // self.nelx) % self.nely] + ([e // (self.nelx * self.nely)] if self.dim == 3 else [])
        return np.stack(ijk, axis=0)

    def get_element_position(self, el_idx=None):
        """Centre coordinates (dim, #elements) of element number(s)."""
        ijk = self.get_element_indices(el_idx)
        return ((self.origin + self.element_size / 2)[: self.dim] + self.element_size[: self.dim] * ijk.T).T

    def get_elemconnectivity(self, i, j, k=0):
        """Node numbers (..., nodes per element) of the elements with indices (i, j, k), in the local node order."""
        i, j, k = np.asarray(i), np.asarray(j), np.asarray(k)
        return np.stack([self.get_nodenumber(i + (a & 1), j + ((a >> 1) & 1), k + ((a >> 2) & 1))
                         for a in range(self.elemnodes)], axis=-1)

    def get_rigid_body_modes(self):
        """Translations and rotations about the origin, (dim * #nodes, dim (dim + 1) / 2): x, y[, z]
        translations, then [Rx, Ry,] Rz."""
        d = self.dim
        rbm = np.zeros((self.nnodes * d, d * (d + 1) // 2))
        for c in range(d):
            rbm[c::d, c] = 1.0
        x = self.get_node_position()
        if d == 3:
            rbm[1::d, -3], rbm[2::d, -3] = x[2], -x[1]
            rbm[0::d, -2], rbm[2::d, -2] = x[2], -x[0]
        rbm[0::d, -1], rbm[1::d, -1] = -x[1], x[0]
        return rbm

    def eval_shape_fun(self, pos):
        """Bilinear / trilinear shape functions at local coordinates pos in [-h/2, h/2]:
        N_a = prod_c (h_c / 2 + s_ac pos_c) / V, s_ac the corner signs of local node a."""
        h = self.element_size[: self.dim]
        v = np.prod(h)
        if not v > 0.0:
            raise ValueError("Element volume needs to be positive")
        n = np.ones(self.elemnodes) / v
        for c in range(self.dim):
            n = n * np.array([h[c] / 2 + sg[c] * pos[c] for sg in self.node_numbering])
        return n

    def eval_shape_fun_der(self, pos):
        """dN_a/dx_c (dim, nodes per element) at local coordinates pos."""
        h = self.element_size[: self.dim]
        v = np.prod(h)
        if not v > 0.0:
            raise ValueError("Element volume needs to be positive")
        dn = np.ones((self.dim, self.elemnodes)) / v
        for c in range(self.dim):
            for o in range(self.dim):
                if o != c:
                    dn[c] = dn[c] * np.array([h[o] / 2 + sg[o] * pos[o] for sg in self.node_numbering])
            dn[c] = dn[c] * np.array([sg[c] for sg in self.node_numbering])
        return dn

    def get_elemnumber(self, eli, elj, elk=0):
        return (np.asarray(elk) * self.nely + elj) * self.nelx + eli

    def get_nodenumber(self, nodi, nodj, nodk=0):
        return (np.asarray(nodk) * (self.nely + 1) + nodj) * (self.nelx + 1) + nodi

    def get_dofnumber(self, nod_idx, dof_idx=None, ndof=None):
        ndof = self.dim if ndof is None else ndof
        dof_idx = np.arange(ndof) if dof_idx is None else np.asarray(dof_idx)
        nod_idx = np.asarray(nod_idx)
        if dof_idx.ndim == 0 or nod_idx.ndim == 0:
            return nod_idx * ndof + dof_idx
        return nod_idx[..., None] * ndof + dof_idx

    @property
    def conn(self):
        e = np.arange(self.nel)
        i, j, k = e % self.nelx, (e // self.nelx) % self.nely, e // (self.nelx * self.nely)
        return np.stack([self.get_nodenumber(i + (a & 1), j + ((a >> 1) & 1), k + ((a >> 2) & 1))
                         for a in range(self.elemnodes)], axis=-1)

    def get_dofconnectivity(self, ndof):
        c = self.conn
        return (c[:, :, None] * ndof + np.arange(ndof)).reshape(c.shape[0], -1)

    def write_to_vti(self, vectors: dict, filename="out.vti", scale=1.0, wait=True):
        """Write `vectors` (numpy arrays or CUDA tensors of size a multiple of nel or nnodes) to a Paraview VTI
        file, as pyMOTO's VoxelDomain.write_to_vti (pymoto/common/domain.py:452-604).  With wait=False the
        device-to-host copies are queued on the current stream and the file is written by a background
        thread (pymoto_gb300.vti.flush() waits for it)."""
        from .vti import write_to_vti
        return write_to_vti(self, vectors, filename, scale, wait=wait)

    def coarse(self):
        return VoxelDomain(self.nelx // 2, self.nely // 2, self.nelz // 2, 2 * self.unitx, 2 * self.unity,
                           2 * self.unitz)


def grid_of(domain):
    """(nelx, nely, nelz) of a pymoto_gb300 or pyMOTO VoxelDomain."""
    return int(domain.nelx), int(domain.nely), int(domain.nelz or 0)
