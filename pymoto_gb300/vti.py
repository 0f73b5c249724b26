"""Paraview image-data (VTI) output of design and state fields, from device buffers.

The file is the one pyMOTO's VoxelDomain.write_to_vti writes (pymoto/common/domain.py:452-604): XML
`ImageData` over the element grid, fields sorted into point data (size a multiple of nnodes) and cell data
(size a multiple of nel), each field a binary `Float32` `DataArray` in base64 preceded by the base64 of an
unsigned 64-bit block length (the length of the encoded block, as the reference writes it), 2D two-component
point vectors padded to three components, block vectors (2-D arrays) split into numbered fields.

What differs is where the time goes: CUDA tensors are copied to pinned host buffers on the current stream and
a background thread waits for the copies and encodes and writes the file, so a design loop that writes a
snapshot every iteration does not wait for the file system.  `flush()` waits for the writes.
"""
import atexit
import base64
import os
import struct
import sys
import threading
import warnings

from pathlib import Path

import numpy as np
import torch

from .core import Module


def _host_array(v):
    if isinstance(v, torch.Tensor):
        return v.detach().cpu().numpy()
    return np.asarray(v)


def _origin_and_spacing(domain, scale):
    origin = np.asarray(getattr(domain, "origin", np.zeros(3)))
    size = np.array([domain.unitx, domain.unity, domain.unitz])
    return [origin[i] * scale for i in range(3)], size[0:3] * scale


def _data_array(name, ncomp, values):
    """One binary Float32 DataArray: header, base64 length block, base64 data."""
    enc = base64.b64encode(np.ascontiguousarray(values, dtype=np.float32))
    order = "<" if sys.byteorder == "little" else ">"
    head = (f'<DataArray type="Float32" Name="{name}" NumberOfComponents="{ncomp}" format="binary">\n').encode()
    return head + base64.b64encode(struct.pack(order + "Q", len(enc))) + enc + b"\n</DataArray>\n"


def _arrays(domain, fields, nunits, point):
    """(name, components, float32 values) of each field of one kind (point or cell data)."""
    out = []
    dim = 2 if not domain.nelz else 3
    for key, vec in fields.items():
        if vec.ndim > 2:
            raise ValueError("only 1D and 2D arrays can be written")
        ax = next((i for i, s in enumerate(vec.shape) if s % nunits == 0), None)
        if ax is None:
            raise ValueError(f"no axis of {key} (shape {vec.shape}) is a multiple of {nunits}")
        ncomp = vec.shape[ax] // nunits
        pad = point and ncomp == 2 and dim == 2
        nvec = 1 if vec.ndim == 1 else vec.shape[(ax + 1) % 2]
        digits = int(np.ceil(np.log10(nvec))) if nvec > 1 else 0
        for i in range(nvec):
            name = key
            vi = vec
            if nvec > 1:
                name += f"({i:0{digits}d})" if point else f"({i})"
                sl = [slice(None), slice(None)]
                sl[(ax + 1) % 2] = i
                vi = vec[tuple(sl)]
            vi = vi.reshape(-1)
            parts = [(vi.real, name + "(real)"), (vi.imag, name + "(imag)")] if np.iscomplexobj(vi) else [(vi, name)]
            for v, nm in parts:
                v = v.astype(np.float32)
                if pad:
                    p3 = np.zeros(3 * (v.size // 2), dtype=np.float32)
                    p3[0::3], p3[1::3] = v[0::2], v[1::2]
                    v = p3
                out.append((nm, 3 if pad else ncomp, v))
    return out


def encode_vti(domain, vectors, scale=1.0):
    """The bytes of the VTI file of `vectors` (name -> array of size a multiple of nel or nnodes), or None
    when nothing can be written."""
    nel = domain.nelx * domain.nely * max(domain.nelz, 1)
    nnodes = (domain.nelx + 1) * (domain.nely + 1) * (domain.nelz + 1)
    point, cell = {}, {}
    for key, vec in vectors.items():
        a = _host_array(vec)
        if a.size % nel == 0:
            cell[key] = a
        elif a.size % nnodes == 0:
            point[key] = a
        else:
            warnings.warn(f"Vector {key} is neither cell- nor point-data. Skipping vector...")
    if not point and not cell:
        return None
    origin, spacing = _origin_and_spacing(domain, scale)
    ext = f"0 {domain.nelx} 0 {domain.nely} 0 {domain.nelz}"
    order = "LittleEndian" if sys.byteorder == "little" else "BigEndian"
    b = [b'<?xml version="1.0"?>\n',
         f'<VTKFile type="ImageData" version="0.1" header_type="UInt64" byte_order="{order}">\n'.encode(),
         f'<ImageData WholeExtent="{ext}"'.encode(),
         f' Origin="{origin[0]} {origin[1]} {origin[2]}"'.encode(),
         f' Spacing="{spacing[0]} {spacing[1]} {spacing[2]}">\n'.encode(),
         f'<Piece Extent="{ext}">\n'.encode()]
    for tag, fields, units, is_point in ((b"PointData", point, nnodes, True), (b"CellData", cell, nel, False)):
        if fields:
            b.append(b"<" + tag + b">\n")
            b += [_data_array(nm, nc, v) for nm, nc, v in _arrays(domain, fields, units, is_point)]
            b.append(b"</" + tag + b">\n")
    b += [b"</Piece>\n", b"</ImageData>\n", b"</VTKFile>"]
    return b"".join(b)


class VTIWriter:
    """Asynchronous writer: write(domain, vectors, filename) queues the device-to-host copies on the current
    stream and returns; a background thread waits for them and writes the file."""

    def __init__(self):
        self._threads = []
        self._errors = []
        atexit.register(self.flush)

    def write(self, domain, vectors, filename="out.vti", scale=1.0):
        self._raise_pending()
        if ".vti" not in os.path.splitext(filename)[-1].lower():
            filename += ".vti"
        staged, event = {}, None
        for key, v in vectors.items():
            if isinstance(v, torch.Tensor) and v.is_cuda:
                h = torch.empty(v.shape, dtype=v.dtype, pin_memory=True)
                h.copy_(v, non_blocking=True)
                staged[key] = h
            else:
                staged[key] = np.array(_host_array(v), copy=True)
        if any(isinstance(v, torch.Tensor) for v in staged.values()):
            event = torch.cuda.Event()
            event.record()

        def work():
            try:
                if event is not None:
                    event.synchronize()
                data = encode_vti(domain, staged, scale)
                if data is None:
                    warnings.warn(f"Nothing to write to {filename}. Skipping file...")
                    return
                with open(filename, "wb") as fh:
                    fh.write(data)
            except Exception as e:   # reported by the next write() or flush()
                self._errors.append((filename, e))

        t = threading.Thread(target=work, daemon=True)
        t.start()
        self._threads = [x for x in self._threads if x.is_alive()] + [t]
        return t

    def flush(self):
        """Wait for the files written so far; raise if one of them could not be written."""
        for t in self._threads:
            t.join()
        self._threads = []
        self._raise_pending()

    def _raise_pending(self):
        if self._errors:
            (fn, e), self._errors = self._errors[0], []
            raise RuntimeError(f"could not write {fn}: {e}") from e


_default = VTIWriter()


def write_to_vti(domain, vectors, filename="out.vti", scale=1.0, wait=False):
    """pyMOTO's VoxelDomain.write_to_vti for pymoto_gb300 (and pyMOTO) domains; asynchronous unless `wait`."""
    t = _default.write(domain, vectors, filename, scale)
    if wait:
        t.join()
        _default._raise_pending()
    return t


def flush():
    _default.flush()


class WriteToVTI(Module):
    """pyMOTO's WriteToVTI module (pymoto/modules/io.py:286-348): writes its input signals, named by their tags,
    to `saveto` (numbered `name.0000.vti`, ... unless `overwrite`) every `interval` responses.  The files are
    written by a background thread from pinned host copies of the device states; `flush()` waits for them."""

    def __init__(self, domain, saveto: str, overwrite: bool = False, scale=1.0, interval=1):
        self.domain = domain
        self.saveto = saveto
        Path(saveto).parent.mkdir(parents=True, exist_ok=True)
        ext = os.path.splitext(saveto)[-1].lower()
        if ext not in (".vti",):
            raise ValueError(f"Extension `{ext}` is not supported. Supported extensions are ('.vti',) ")
        self.iter = 0
        self.scale = scale
        self.overwrite = overwrite
        self.interval = interval
        self.writer = VTIWriter()

    def __call__(self, *args):
        if self.iter % self.interval != 0:
            self.iter += 1
            return
        if len(args) == 0:
            raise ValueError("Nothing to write to VTI file")
        data = {}
        for i, x in enumerate(args):
            name = f"inp{i:d}"
            if self.sig_in is not None:
                name = getattr(self.sig_in[i], "tag", name)
            data[name] = x
        root, ext = os.path.splitext(self.saveto)
        fname = root + ext if self.overwrite else f"{root}.{self.iter:04d}{ext}"
        self.writer.write(self.domain, data, fname, self.scale)
        self.iter += 1

    def flush(self):
        self.writer.flush()
