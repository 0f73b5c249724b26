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
