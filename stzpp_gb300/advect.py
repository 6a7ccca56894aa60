"""The quasi-static advection step of shear_sim_3d on the GPU.

Python binding of ``stz_mg_advection_step`` (include/stz_mg.h): the per-step update of
the stresses and the effective temperature before the projection solve
(shear_sim_3d::advection_step, src/shear_sim_3d.cpp:393-525), on CUDA tensors
that hold the reference's ghosted grid ((nx+4) x (ny+4) x (nz+4) points, x
fastest), one float64 tensor per Field member.
"""
from __future__ import annotations

import ctypes

from . import mg as _mg

INPUTS = ("u", "v", "w", "s11", "s12", "s13", "s22", "s23", "s33", "chi")
OUTPUTS = ("ad_dpl", "sbar", "cs11", "cs12", "cs13", "cs22", "cs23", "cs33", "cchi")
PARAMS = ("mu", "sy", "tau0", "eps0", "c0", "delta", "omega", "bath_temp", "chi_inf", "ez", "diff_l")
NGHOST = 2


class AdvParams(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double)] + \
               [(n, ctypes.c_double) for n in PARAMS]


class AdvFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in INPUTS + OUTPUTS + ("work",)]


def grid_points(nx, ny, nz):
    """Points of the ghosted grid."""
    return (nx + 2 * NGHOST) * (ny + 2 * NGHOST) * (nz + 2 * NGHOST)


def work_size(nx, ny, nz):
    """Doubles of scratch the step needs."""
    return 2 * grid_points(nx, ny, nz) + 2


def advection_step(fields, dims, spacing, params, dt, work=None, stream=None, wait=True):
    """One advection step in place on the CUDA float64 tensors ``fields``
    (names INPUTS + OUTPUTS, each of grid_points(*dims) elements).  ``params``
    maps the STZ parameter names PARAMS to values.  With ``wait`` the call
    synchronises and returns whether some point reached the yield stress;
    otherwise it returns None and stays asynchronous on ``stream`` (a
    torch.cuda.Stream, default: the current stream)."""
    import torch
    nx, ny, nz = dims
    n = grid_points(nx, ny, nz)
    for name in INPUTS + OUTPUTS:
        t = fields[name]
        if not (t.is_cuda and t.dtype == torch.float64 and t.is_contiguous() and t.numel() == n):
            raise ValueError(f"field {name}: expected a contiguous float64 CUDA tensor of {n} elements")
    if work is None:
        work = torch.empty(work_size(nx, ny, nz), dtype=torch.float64, device=fields["u"].device)
    p = AdvParams(nx, ny, nz, *spacing, *[float(params[k]) for k in PARAMS])
    f = AdvFields(*[fields[k].data_ptr() for k in INPUTS + OUTPUTS], work.data_ptr())
    st = (stream or torch.cuda.current_stream()).cuda_stream
    y = ctypes.c_int(0)
    lib = _mg.load_library()
    rc = lib.stz_mg_advection_step(ctypes.byref(p), ctypes.byref(f), float(dt), ctypes.c_void_p(st),
                                   ctypes.byref(y) if wait else None)
    _mg._check(rc)
    return bool(y.value) if wait else None


CUBE_MEMBERS = ("u", "v", "w", "s11", "s12", "s13", "s22", "s23", "s33", "chi", "xi_x", "xi_y", "xi_z")


class CubeFields(ctypes.Structure):
    _fields_ = [(n, ctypes.c_void_p) for n in CUBE_MEMBERS]


def _cube_fields(fields):
    return CubeFields(*[fields[k].data_ptr() if fields.get(k) is not None else None for k in CUBE_MEMBERS])


def cube_values(fields, dims, mode, stream=None):
    """shear_sim_3d::output_cube's values of Field member `mode` (0-15, as
    Field::fval) on the device: a float32 CUDA tensor, x slowest, z fastest,
    the node-based members with the top z node.  ``fields``: CUDA float64
    tensors over the ghosted grid (members the mode does not read may be
    missing)."""
    import torch
    nx, ny, nz = dims
    zsize = nz + 1 if (mode <= 2 or mode >= 13) else nz
    out = torch.empty(nx * ny * zsize, dtype=torch.float32, device=next(iter(fields.values())).device)
    f = _cube_fields(fields)
    st = (stream or torch.cuda.current_stream()).cuda_stream
    _mg._check(_mg.load_library().stz_mg_cube_values(ctypes.byref(f), nx, ny, nz, mode,
                                                     ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(st)))
    return out


def output_cube(fields, dims, mode, directory, prefix, frame):
    """Append Field member `mode` to <directory>/<prefix>_grid.<frame> in the
    reference's cube format (shear_sim_3d::output_cube)."""
    import os
    import torch
    torch.cuda.current_stream().synchronize()
    f = _cube_fields(fields)
    _mg._check(_mg.load_library().stz_mg_output_cube(ctypes.byref(f), *dims, mode, os.fsencode(directory),
                                                     prefix.encode(), frame))
