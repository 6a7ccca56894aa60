"""The reference's output file formats restated with numpy, for tests.

Test infrastructure only.  ``slice_file`` gives the bytes that
region::output_internal (mg_3d_template/region.cc:3135-3202) writes for a
z-slice of a vec3 field of one process (output_x, output_r, output_residual,
region.cc:3062-3120, whose values pass through vec3::operator double, the
squared magnitude, src/vec3.hh:110-112); ``cube_file`` the bytes one
shear_sim_3d::output_cube call appends (src/shear_sim_3d.cpp:1961-2158; the
values are oracle.advect.cube_values).
"""
from __future__ import annotations

import numpy as np


def vec3_sq(v):
    """vec3::operator double, x*x + y*y + z*z in that order."""
    return (v[..., 0] * v[..., 0] + v[..., 1] * v[..., 1]) + v[..., 2] * v[..., 2]


def slice_file(field, dims, k, box, quartic=False):
    """Bytes of the z-slice k of a (npts, 3) vec3 field in natural order (x
    fastest) on an m x n x o grid; quartic: output_residual's |r|^2 |r|^2."""
    m, n, o = dims
    ax, bx, ay, by = box
    v = vec3_sq(np.asarray(field, dtype=np.float64).reshape(o, n, m, 3)[k])
    if quartic:
        v = v * v
    dx, dy = (bx - ax) / (m - 1), (by - ay) / (n - 1)
    head = np.array([m] + [ax + dx * i for i in range(m)], dtype=np.float64).astype(np.float32)
    rows = [np.concatenate([np.array([ay + dy * j]).astype(np.float32), v[j].astype(np.float32)]) for j in range(n)]
    return head.tobytes() + b"".join(r.tobytes() for r in rows)


def cube_file(fields, nx, ny, nz, mode):
    """Bytes one output_cube call appends for Field member `mode`."""
    from oracle import advect
    return advect.cube_values(fields, nx, ny, nz, mode).tobytes()
