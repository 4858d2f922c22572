"""Host-side mirror of the reference's interface for the .grad path.

* :func:`steepest_lstar` / :func:`lower_star_grad` -- the complete .grad of
  ``steepest_lstar`` (3D) or of ``Accurate2D::DiscreteGradientBuilder`` without saddle
  streamlines (2D), computed by libmsc_gpu.so.  Accepts a CUDA ``torch.Tensor``
  (device-resident, enqueued on the current stream) or a ``numpy`` array (host
  buffers; copies in and out through the C ABI).
* :class:`TopologicalRegularGrid3D` / :class:`TopologicalRegularGrid2D` -- the index
  algebra of gi_topological_regular_grid.h (cellid2Coords :1268, coords2Cellid :1274,
  dimension :1314, boundaryValue :1291, VertexNumberFromCellID :1337), vectorised.
* :class:`DiscreteGradientLabeling` -- the per-cell byte accessors of
  gi_discrete_gradient_labeling.h (getAssigned :71, getPair :87, getCritical :99,
  getDimAscMan :114, outputToFile :200, load_from_file :229).
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

from . import _lib


def _is_torch(x) -> bool:
    return type(x).__module__.startswith("torch")


def _shape_dims(shape):
    """numpy/torch shape (Z, Y, X) or (Y, X) -> reference dims (X, Y, Z) / (X, Y)."""
    if len(shape) not in (2, 3):
        raise ValueError(f"expected a 2D or 3D volume, got shape {tuple(shape)}")
    return tuple(int(s) for s in shape[::-1])


def num_cells(dims) -> int:
    lib = _lib.load()
    fn = lib.msc_num_cells_3d if len(dims) == 3 else lib.msc_num_cells_2d
    n = fn(_lib.dims_arg(dims))
    if n < 0:
        raise ValueError(f"invalid dims {dims}")
    return int(n)


def _device_call(name3, name2, f, out):
    import torch

    if f.dtype != torch.float32:
        raise TypeError("f must be float32")
    f = f.contiguous()
    dims = _shape_dims(f.shape)
    n = num_cells(dims)
    if out is None:
        out = torch.empty(n, dtype=torch.uint8, device=f.device)
    elif out.dtype != torch.uint8 or out.numel() != n or not out.is_contiguous() or out.device != f.device:
        raise ValueError("out must be a contiguous uint8 tensor of num_cells bytes on f's device")
    lib = _lib.load()
    name = name3 if len(dims) == 3 else name2
    stream = torch.cuda.current_stream(f.device).cuda_stream
    with torch.cuda.device(f.device):
        rc = getattr(lib, name)(ctypes.c_void_p(f.data_ptr()), _lib.dims_arg(dims),
                                ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(stream))
    _lib.check(rc, name)
    return out


def lower_star_grad(f, out=None):
    """The complete .grad (one byte per cell, x fastest) of a float32 volume."""
    if _is_torch(f):
        if not f.is_cuda:
            f = f.numpy()
        else:
            return _device_call("msc_lower_star_grad_3d", "msc_lower_star_grad_2d", f, out)
    f = np.ascontiguousarray(f, dtype=np.float32)
    dims = _shape_dims(f.shape)
    n = num_cells(dims)
    if out is None:
        out = np.empty(n, dtype=np.uint8)
    lib = _lib.load()
    name = "msc_steepest_lstar_host" if len(dims) == 3 else "msc_lower_star_grad_2d_host"
    rc = getattr(lib, name)(f.ctypes.data_as(ctypes.c_void_p), _lib.dims_arg(dims),
                            out.ctypes.data_as(ctypes.c_void_p))
    _lib.check(rc, name)
    return out


def lower_star_grad_batch(volumes, outs=None, threads: int = 0):
    """The .grad of many 3D CUDA float32 volumes of different sizes in shared launches
    (msc_lower_star_grad_batch_3d).  Returns the list of uint8 tensors."""
    import torch

    vols = [v.contiguous() for v in volumes]
    if not vols:
        return []
    dev = vols[0].device
    dims = [_shape_dims(v.shape) for v in vols]
    if any(len(d) != 3 for d in dims):
        raise ValueError("batched volumes must be 3D")
    if outs is None:
        outs = [torch.empty(num_cells(d), dtype=torch.uint8, device=dev) for d in dims]
    n = len(vols)
    fp = (ctypes.c_void_p * n)(*[v.data_ptr() for v in vols])
    gp = (ctypes.c_void_p * n)(*[o.data_ptr() for o in outs])
    dd = (ctypes.c_int64 * (3 * n))(*[x for d in dims for x in d])
    lib = _lib.load()
    stream = torch.cuda.current_stream(dev).cuda_stream
    with torch.cuda.device(dev):
        rc = lib.msc_lower_star_grad_batch_3d(n, ctypes.cast(fp, ctypes.c_void_p), dd,
                                              ctypes.cast(gp, ctypes.c_void_p), ctypes.c_void_p(stream))
    _lib.check(rc, "msc_lower_star_grad_batch_3d")
    return outs


def steepest_lstar(f, out=None):
    """steepest_lstar's .grad for a 3D volume (numpy host array or CUDA tensor)."""
    if len(f.shape) != 3:
        raise ValueError("steepest_lstar takes a 3D volume")
    return lower_star_grad(f, out)


def lower_star_pairs(f, out=None):
    """Stage 1 only (CUDA tensors): pairs, flag and the ascending-manifold roots."""
    return _device_call("msc_lower_star_pairs_3d", "msc_lower_star_pairs_2d", f, out)


def ascending_manifold_dims(grad, dims) -> int:
    """Stage 2 only (CUDA uint8 tensor, in place); returns the number of tile passes."""
    import torch

    lib = _lib.load()
    name = "msc_ascending_manifold_dims_3d" if len(dims) == 3 else "msc_ascending_manifold_dims_2d"
    passes = ctypes.c_int(0)
    stream = torch.cuda.current_stream(grad.device).cuda_stream
    with torch.cuda.device(grad.device):
        rc = getattr(lib, name)(ctypes.c_void_p(grad.data_ptr()), _lib.dims_arg(dims),
                                ctypes.c_void_p(stream), ctypes.byref(passes))
    _lib.check(rc, name)
    return passes.value


def integrated_labels(f, grad, error_threshold=1e-4, gradient_threshold=None, iteration_limit=4000,
                      max_step=0.25, presimp_threshold=0.0, ascending=True, descending=True, stages=False,
                      precision=0):
    """ondemandaccurate's ascending / descending 3-manifold labels of a device volume.

    ``f``: CUDA float32 (Z, Y, X); ``grad``: its .grad from :func:`lower_star_grad`.
    ``gradient_threshold`` defaults to 1e-6 of max|f|.  ``precision`` 0 re-decides
    boundary vertices in FP32 and the ambiguous ones in FP64; 1 re-decides all of them
    in FP64.  Returns a dict with "asc" and/or "dsc" int32 tensors (a label is the
    vertex id of the region's extremum, -1 none), "stats" (boundary re-decisions and
    FP64 ones per direction, and the advection iterations of each stage) and, with
    ``stages``, the terminal / integrated labels of each direction."""
    import torch

    if not (f.is_cuda and grad.is_cuda):
        raise ValueError("integrated_labels takes CUDA tensors")
    f = f.contiguous()
    dims = _shape_dims(f.shape)
    if len(dims) != 3:
        raise ValueError("integrated labels are defined for 3D volumes")
    if gradient_threshold is None:
        gradient_threshold = 1e-6 * float(f.abs().max())
    p = _lib.IntegParams(error_threshold, gradient_threshold, iteration_limit, max_step, presimp_threshold,
                         int(precision))
    n = f.numel()
    asc = torch.empty(n, dtype=torch.int32, device=f.device) if ascending else None
    dsc = torch.empty(n, dtype=torch.int32, device=f.device) if descending else None
    st = torch.empty(4 * n, dtype=torch.int32, device=f.device) if stages else None
    lib = _lib.load()
    stream = torch.cuda.current_stream(f.device).cuda_stream
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    with torch.cuda.device(f.device):
        if stages:
            rc = lib.msc_integrated_labels_3d_stages(ptr(f), ptr(grad), _lib.dims_arg(dims), ctypes.byref(p),
                                                     ptr(asc), ptr(dsc), ptr(st), ctypes.c_void_p(stream))
        else:
            rc = lib.msc_integrated_labels_3d(ptr(f), ptr(grad), _lib.dims_arg(dims), ctypes.byref(p), ptr(asc),
                                              ptr(dsc), ctypes.c_void_p(stream))
    _lib.check(rc, "msc_integrated_labels_3d")
    stats = (ctypes.c_int64 * 4)()
    lib.msc_labels_last_stats(stats)
    it = (ctypes.c_int64 * 6)()
    lib.msc_labels_last_iterations(it)
    sd = {"asc_redecided": stats[0], "asc_fp64": stats[1], "dsc_redecided": stats[2], "dsc_fp64": stats[3]}
    sd.update({f"{d}_iterations_{k}": it[3 * i + j] for i, d in enumerate(("asc", "dsc"))
               for j, k in enumerate(("first_pass", "fp32", "fp64"))})
    out = {"stats": sd}
    if asc is not None:
        out["asc"] = asc
    if dsc is not None:
        out["dsc"] = dsc
    if stages:
        for i, k in enumerate(("asc_terminal", "asc_integrated", "dsc_terminal", "dsc_integrated")):
            out[k] = st[i * n:(i + 1) * n]
    return out


def conforming_grad(f, grad, labels_asc=None, labels_dsc=None, restriction=False):
    """ondemandaccurate's accurate 3-manifold .grad (msc_conforming_grad_3d): ``grad`` (the
    base .grad of :func:`lower_star_grad`, CUDA uint8) is re-paired in place around the
    boundaries of the final labels ``labels_asc`` / ``labels_dsc`` (CUDA int32, either
    may be None).  Returns the number of re-paired vertices, and with ``restriction``
    also the restriction byte of every cell."""
    import torch

    f = f.contiguous()
    dims = _shape_dims(f.shape)
    if len(dims) != 3 or not (f.is_cuda and grad.is_cuda):
        raise ValueError("conforming_grad takes a CUDA 3D volume and its .grad")
    rl = torch.empty(num_cells(dims), dtype=torch.uint8, device=f.device) if restriction else None
    touched = ctypes.c_int64(0)
    ptr = lambda t: ctypes.c_void_p(t.contiguous().data_ptr()) if t is not None else None  # noqa: E731
    lib = _lib.load()
    stream = torch.cuda.current_stream(f.device).cuda_stream
    with torch.cuda.device(f.device):
        rc = lib.msc_conforming_grad_3d(ptr(f), ptr(labels_asc), ptr(labels_dsc), _lib.dims_arg(dims), ptr(grad),
                                        ptr(rl), ctypes.byref(touched), ctypes.c_void_p(stream))
    _lib.check(rc, "msc_conforming_grad_3d")
    return (touched.value, rl) if restriction else touched.value


def ms_graph(grad, f, build_arcs=(1, 0, 1)):
    """MorseSmaleComplexBasic::ComputeFromGrad without arc geometry on a device .grad
    (msc_ms_graph_3d): the critical cells as nodes and the traced V-paths as arcs.
    ``grad``: CUDA uint8 .grad of ``f`` (CUDA float32 (Z, Y, X)); ``build_arcs``: the
    reference's SetBuildArcs flags (arcs from 1-saddles, 2-saddles, maxima; extractmsc
    uses (1, 0, 1)).  Returns a dict of CUDA tensors: node_cell (int64), node_value
    (float32), node_dim / node_boundary (uint8), arc_lower / arc_upper (int32 node
    indices) and arc_persistence (float32)."""
    import torch

    f = f.contiguous()
    dims = _shape_dims(f.shape)
    if len(dims) != 3 or not (f.is_cuda and grad.is_cuda) or grad.numel() != num_cells(dims):
        raise ValueError("ms_graph takes a CUDA 3D volume and its .grad")
    lib = _lib.load()
    dev = f.device
    stream = torch.cuda.current_stream(dev).cuda_stream
    b = (ctypes.c_int * 3)(*[int(x) for x in build_arcs])
    counts = (ctypes.c_int64 * 2)()
    ptr = lambda t: ctypes.c_void_p(t.data_ptr())  # noqa: E731
    with torch.cuda.device(dev):
        rc = lib.msc_ms_graph_3d(ptr(grad), ptr(f), _lib.dims_arg(dims), b, 0, None, None, None, None, 0, None, None,
                                 None, counts, ctypes.c_void_p(stream))
        _lib.check(rc, "msc_ms_graph_3d")
        nn, na = counts[0], counts[1]
        out = {"node_cell": torch.empty(nn, dtype=torch.int64, device=dev),
               "node_value": torch.empty(nn, dtype=torch.float32, device=dev),
               "node_dim": torch.empty(nn, dtype=torch.uint8, device=dev),
               "node_boundary": torch.empty(nn, dtype=torch.uint8, device=dev),
               "arc_lower": torch.empty(na, dtype=torch.int32, device=dev),
               "arc_upper": torch.empty(na, dtype=torch.int32, device=dev),
               "arc_persistence": torch.empty(na, dtype=torch.float32, device=dev)}
        rc = lib.msc_ms_graph_3d(ptr(grad), ptr(f), _lib.dims_arg(dims), b, nn, ptr(out["node_cell"]),
                                 ptr(out["node_value"]), ptr(out["node_dim"]), ptr(out["node_boundary"]), na,
                                 ptr(out["arc_lower"]), ptr(out["arc_upper"]), ptr(out["arc_persistence"]), counts,
                                 ctypes.c_void_p(stream))
        _lib.check(rc, "msc_ms_graph_3d")
    return out


def saddle_lines(f, grad, cells=None, which=3, zeroed=None, error_threshold=1e-4, gradient_threshold=None,
                 iteration_limit=4000, max_step=0.25):
    """ondemandaccurate's saddle streamline digitizers (needASC1 / needDSC1) on a device
    volume (msc_saddle_lines_3d): ``which`` bit 0 the ascending lines from the 2-saddles
    (label 4 on hexes and faces), bit 1 the descending lines from the 1-saddles (label 5
    on vertices and edges).  ``cells``: CUDA uint8, one byte per cell (zeros when not
    given), updated in a copy; ``zeroed``: CUDA int32/uint32 bitmap of vertices with a
    zero gradient, or None.  Returns (cells, stats) with stats = (streamlines, recorded
    voxel steps, kept voxel steps, rounds)."""
    import torch

    if not (f.is_cuda and grad.is_cuda):
        raise ValueError("saddle_lines takes CUDA tensors")
    f = f.contiguous()
    dims = _shape_dims(f.shape)
    if len(dims) != 3 or grad.numel() != num_cells(dims):
        raise ValueError("saddle_lines takes a 3D volume and its .grad")
    if gradient_threshold is None:
        gradient_threshold = 1e-6 * float(f.abs().max())
    out = (torch.zeros(grad.numel(), dtype=torch.uint8, device=f.device) if cells is None
           else cells.to(device=f.device, dtype=torch.uint8).contiguous().clone())
    if zeroed is not None:
        zeroed = zeroed.contiguous()
        if not zeroed.is_cuda or zeroed.element_size() != 4 or zeroed.numel() * 32 < f.numel():
            raise ValueError("zeroed must be a CUDA 32-bit bitmap of at least one bit per vertex")
    p = _lib.IntegParams(error_threshold, gradient_threshold, iteration_limit, max_step, 0.0, 0)
    stats = (ctypes.c_int64 * 4)()
    lib = _lib.load()
    stream = torch.cuda.current_stream(f.device).cuda_stream
    ptr = lambda t: ctypes.c_void_p(t.data_ptr()) if t is not None else None  # noqa: E731
    with torch.cuda.device(f.device):
        rc = lib.msc_saddle_lines_3d(ptr(f), ptr(grad), ptr(zeroed), _lib.dims_arg(dims), int(which), ctypes.byref(p),
                                     ptr(out), stats, ctypes.c_void_p(stream))
    _lib.check(rc, "msc_saddle_lines_3d")
    return out, tuple(int(x) for x in stats)


def clean_regions(f, labels, direction):
    """IsolatedCCRegionRemoverNEW on device labels (msc_clean_regions_3d): ``direction``
    -1 for ascending labels (lowest value first), +1 for descending ones.  ``f``: CUDA
    float32 (Z, Y, X); ``labels``: CUDA int32 per vertex, -1 = none.  Returns the cleaned
    labels as a new tensor."""
    import torch

    if not (f.is_cuda and labels.is_cuda):
        raise ValueError("clean_regions takes CUDA tensors")
    f = f.contiguous()
    labels = labels.contiguous().view(-1)
    dims = _shape_dims(f.shape)
    if len(dims) != 3 or labels.numel() != f.numel() or labels.dtype != torch.int32:
        raise ValueError("clean_regions takes a 3D volume and one int32 label per vertex")
    out = torch.empty_like(labels)
    lib = _lib.load()
    stream = torch.cuda.current_stream(f.device).cuda_stream
    with torch.cuda.device(f.device):
        rc = lib.msc_clean_regions_3d(ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(labels.data_ptr()),
                                      _lib.dims_arg(dims), int(direction), ctypes.c_void_p(out.data_ptr()),
                                      ctypes.c_void_p(stream))
    _lib.check(rc, "msc_clean_regions_3d")
    return out


def integrated_labels_batch(volumes, grads, threads: int = 4, **kwargs):
    """integrated_labels of many volumes, `threads` at a time on their own CUDA streams
    (each call synchronises only its own stream, so the volumes overlap on the GPU)."""
    import concurrent.futures as cf

    import torch

    def one(i):
        s = torch.cuda.Stream(device=volumes[i].device)
        with torch.cuda.stream(s):
            return integrated_labels(volumes[i], grads[i], **kwargs)

    with cf.ThreadPoolExecutor(max_workers=max(1, threads)) as ex:
        return list(ex.map(one, range(len(volumes))))


class TopologicalRegularGrid3D:
    """Cell-complex index algebra of a non-periodic X x Y x Z vertex grid."""

    nd = 3

    def __init__(self, X: int, Y: int, Z: int):
        self.base = (int(X), int(Y), int(Z))
        self.xyz = tuple(2 * v - 1 for v in self.base)

    def XYZ(self):
        return self.xyz

    def numCells(self) -> int:
        return int(np.prod(self.xyz))

    def maxDim(self) -> int:
        return self.nd

    def cellid2Coords(self, cellid):
        c = np.asarray(cellid, dtype=np.int64)
        dX, dY = self.xyz[0], self.xyz[1]
        out = [c % dX, (c // dX) % dY]
        if self.nd == 3:
            out.append(c // (dX * dY))
        return np.stack(out, axis=-1)

    def coords2Cellid(self, coords):
        c = np.asarray(coords, dtype=np.int64)
        idx = c[..., 0] + c[..., 1] * self.xyz[0]
        if self.nd == 3:
            idx = idx + c[..., 2] * self.xyz[0] * self.xyz[1]
        return idx

    def dimension(self, cellid):
        return (self.cellid2Coords(cellid) & 1).sum(axis=-1)

    def boundaryValue(self, cellid):
        c = self.cellid2Coords(cellid)
        ext = np.asarray(self.xyz[: self.nd])
        return ((c == 0) | (c == ext - 1)).sum(axis=-1)

    def VertexNumberFromCellID(self, cellid):
        c = self.cellid2Coords(cellid) // 2
        v = c[..., 0] + c[..., 1] * self.base[0]
        if self.nd == 3:
            v = v + c[..., 2] * self.base[0] * self.base[1]
        return v

    def adjacency_offsets(self):
        """m_adjacency_offsets: +x, -x, +y, -y[, +z, -z] (gi_topological_regular_grid.h:167-172)."""
        s = [1, self.xyz[0], self.xyz[0] * self.xyz[1]][: self.nd]
        return [o for st in s for o in (st, -st)]


class TopologicalRegularGrid2D(TopologicalRegularGrid3D):
    nd = 2

    def __init__(self, X: int, Y: int):
        self.base = (int(X), int(Y))
        self.xyz = tuple(2 * v - 1 for v in self.base)


class DiscreteGradientLabeling:
    """One GradBitfield byte per cell: assigned:1 flag:1 pair:3 ldir:3 (LSB first)."""

    def __init__(self, mesh: TopologicalRegularGrid3D, data=None):
        self.mesh = mesh
        n = mesh.numCells()
        if data is None:
            data = np.zeros(n, dtype=np.uint8)
        data = np.asarray(data, dtype=np.uint8).reshape(-1)
        if data.size != n:
            raise ValueError(f"expected {n} bytes, got {data.size}")
        self.data = data

    def ClearAllGradient(self):
        self.data[:] = 0

    def getAssigned(self, cellid):
        return self.data[cellid] & 1

    def getCritical(self, cellid):
        return ((self.data[cellid] >> 2) & 7) == 7

    def getPair(self, cellid):
        code = (self.data[cellid] >> 2) & 7
        offs = np.asarray(self.mesh.adjacency_offsets() + [0] * (8 - 2 * self.mesh.nd), dtype=np.int64)
        return np.asarray(cellid, dtype=np.int64) + offs[code]

    def getDimAscMan(self, cellid):
        return self.data[cellid] >> 5

    def getFlag(self, cellid):
        return (self.data[cellid] >> 1) & 1

    def outputToFile(self, filename):
        Path(filename).write_bytes(self.data.tobytes())

    def load_from_file(self, filename) -> bool:
        p = Path(filename)
        if not p.exists():
            return False
        raw = np.fromfile(p, dtype=np.uint8, count=self.mesh.numCells())
        self.data[: raw.size] = raw
        return True

    def critical_counts(self):
        """Critical cells per dimension (count_critical_points,
        gi_topological_gradient_using_algorithms.h:141)."""
        ids = np.nonzero(((self.data >> 2) & 7) == 7)[0]
        dims = self.mesh.dimension(ids)
        return [int((dims == d).sum()) for d in range(self.mesh.nd + 1)]
