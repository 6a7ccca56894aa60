"""Oracle-side problem definition (test infrastructure only).

Numpy restatement of the reference's operator and right-hand side for the
quasi-static projection solve, used by the tests and the bench's CPU leg to
build inputs for the oracles (the compiled reference in ``oracle/_ref`` and
the C restatement in ``oracle/stzmg_oracle.c``).  The product computes the
same quantities itself (host stencil helper, GPU kernels); these functions are
the independent check.

Grid convention (reference region.hh:805 / shear_sim_3d.hh): a periodic
dimension with N cells has N unknown nodes, a Dirichlet dimension has N+1.
Arrays are natural order, x fastest: index p = i + m*(j + n*k), numpy shape
(o, n, m, ...).
"""
from __future__ import annotations

import numpy as np

# Block index of offset (dx,dy,dz): 13 + dx + 3*dy + 9*dz (shear_sim_3d.cpp:224).


def block_index(dx: int, dy: int, dz: int) -> int:
    return 13 + dx + 3 * dy + 9 * dz


def elastic_stencil_const(mu, lam, dx, dy, dz, dt=1.0, kappa=0.0):
    """The shared 27-block stencil and Dirichlet ``fix`` block.

    Follows shear_sim_3d::set_up_stencil_base (src/shear_sim_3d.cpp:215-331)
    block by block, then stencil = -dt*base and
    fix = -dt*2((lam+2mu)/dx^2 + mu/dy^2 + mu/dz^2) I (src/shear_sim_3d.hh:45-55).
    Returns (stencil (27, 9), fix (9,)), blocks row-major (a11, a12, ..., a33).
    """
    base = np.zeros((27, 3, 3))
    lm = lam + mu
    def diag(a, b, c):
        return np.diag([a, b, c])
    def sym(r, c, v):
        m = np.zeros((3, 3)); m[r, c] = v; m[c, r] = v; return m
    kx, ky, kz = kappa / dt / dx / dx, kappa / dt / dy / dy, kappa / dt / dz / dz
    ksum = kappa / dt * (1. / dx / dx + 1. / dy / dy + 1. / dz / dz)
    base[1] = sym(1, 2, lm / 4 / dz / dy)
    base[3] = sym(0, 2, lm / 4 / dx / dz)
    base[4] = diag(mu / dz / dz + kz, mu / dz / dz + kz, (lam + 2 * mu) / dz / dz + kz)
    base[5] = sym(0, 2, -lm / 4 / dx / dz)
    base[7] = sym(1, 2, -lm / 4 / dz / dy)
    base[9] = sym(0, 1, lm / 4 / dx / dy)
    base[10] = diag(mu / dy / dy + ky, (lam + 2 * mu) / dy / dy + ky, mu / dy / dy + ky)
    base[11] = sym(0, 1, -lm / 4 / dx / dy)
    base[12] = diag((lam + 2 * mu) / dx / dx + kx, mu / dx / dx + kx, mu / dx / dx + kx)
    # case 13 keeps the reference's sign placement of the kappa term in a33
    base[13] = diag(-2 * ((lam + 2 * mu) / dx / dx + mu / dy / dy + mu / dz / dz + ksum),
                    -2 * (mu / dx / dx + (lam + 2 * mu) / dy / dy + mu / dz / dz + ksum),
                    -2 * (mu / dx / dx + mu / dy / dy + (lam + 2 * mu) / dz / dz) + ksum)
    base[14] = diag((lam + 2 * mu) / dx / dx + kx, mu / dx / dx + kx, mu / dx / dx + kx)
    base[15] = sym(0, 1, -lm / 4 / dx / dy)
    base[16] = diag(mu / dy / dy + ky, (lam + 2 * mu) / dy / dy + ky, mu / dy / dy + ky)
    base[17] = sym(0, 1, lm / 4 / dx / dy)
    base[19] = sym(1, 2, -lm / 4 / dz / dy)
    base[21] = sym(0, 2, -lm / 4 / dx / dz)
    base[22] = diag(mu / dz / dz + kz, mu / dz / dz + kz, (lam + 2 * mu) / dz / dz + kz)
    base[23] = sym(0, 2, lm / 4 / dx / dz)
    base[25] = sym(1, 2, lm / 4 / dz / dy)
    stencil = (-dt * base).reshape(27, 9)
    fix = (np.eye(3) * (-dt * 2 * ((lam + 2 * mu) / dx / dx + mu / dy / dy + mu / dz / dz))).reshape(9)
    return stencil, fix


def interior_mask(m, n, o, xp, yp, zp):
    """shear_sim_3d::interior (src/shear_sim_3d.hh:378-383) on the node grid."""
    k, j, i = np.meshgrid(np.arange(o), np.arange(n), np.arange(m), indexing="ij")
    ok = np.ones((o, n, m), dtype=bool)
    if not xp:
        ok &= (i != 0) & (i != m - 1)
    if not yp:
        ok &= (j != 0) & (j != n - 1)
    if not zp:
        ok &= (k != 0) & (k != o - 1)
    return ok


def _shift(a, d, axis, periodic):
    """a[index + d] along axis (natural order arrays of shape (o, n, m))."""
    if periodic:
        return np.roll(a, -d, axis=axis)
    out = np.empty_like(a)
    sl_dst = [slice(None)] * a.ndim
    sl_src = [slice(None)] * a.ndim
    L = a.shape[axis]
    if d > 0:
        sl_dst[axis] = slice(0, L - d); sl_src[axis] = slice(d, L)
        out[tuple(sl_dst)] = a[tuple(sl_src)]
        sl_dst[axis] = slice(L - d, L)
        out[tuple(sl_dst)] = np.nan
    elif d < 0:
        sl_dst[axis] = slice(-d, L); sl_src[axis] = slice(0, L + d)
        out[tuple(sl_dst)] = a[tuple(sl_src)]
        sl_dst[axis] = slice(0, -d)
        out[tuple(sl_dst)] = np.nan
    else:
        out[...] = a
    return out


def elastic_stencil_points(mu, lam, dx, dy, dz, periodic, dt=1.0):
    """Per-node stencils (npts, 27, 9) of the variable-coefficient operator.

    The reference only ships a constant-coefficient stencil; this is the
    variable-mu discretisation the product implements (documented in the
    design notes), restated independently here.  Face terms use
    midpoint-averaged coefficients; cross terms d_x(lam d_y v) + d_y(mu d_x v)
    use node values, giving block (+1,+1,0) a12 = (lam[i+1,j] + mu[i,j+1])/(4 dx dy).
    With constant mu, lam it reduces to elastic_stencil_const (kappa = 0).
    Dirichlet rows carry fix = -dt*2((lam+2mu)/dx^2 + mu/dy^2 + mu/dz^2) I of
    the node, in the centre block.
    """
    o, n, m = mu.shape
    xp, yp, zp = periodic
    per = (zp, yp, xp)        # per numpy axis (0: z, 1: y, 2: x)
    h = {2: dx, 1: dy, 0: dz}
    comp_axis = {0: 2, 1: 1, 2: 0}   # component c's own axis in numpy order
    base = np.zeros((o, n, m, 27, 3, 3))
    sh = lambda a, d, ax: _shift(a, d, ax, per[ax])
    # face blocks and centre
    centre = np.zeros((o, n, m, 3))
    for ax in (2, 1, 0):
        for s in (-1, 1):
            mu_f = 0.5 * (mu + sh(mu, s, ax))
            lam_f = 0.5 * (lam + sh(lam, s, ax))
            d = [0, 0, 0]
            d[2 - ax] = s    # (dx, dy, dz) order
            b = block_index(*d)
            for c in range(3):
                coef = (lam_f + 2 * mu_f) if comp_axis[c] == ax else mu_f
                v = coef / (h[ax] * h[ax])
                base[..., b, c, c] = v
                centre[..., c] -= v
    for c in range(3):
        base[..., 13, c, c] = centre[..., c]
    # cross (edge) blocks: for the pair of axes (a, b) in component space
    pairs = [(0, 1), (0, 2), (1, 2)]  # (component r, component c) = (x,y), (x,z), (y,z)
    for (r, c) in pairs:
        ax_r, ax_c = comp_axis[r], comp_axis[c]
        hr, hc = h[ax_r], h[ax_c]
        for sr in (-1, 1):
            for sc in (-1, 1):
                d = [0, 0, 0]
                d[r] = sr
                d[c] = sc
                b = block_index(*d)
                sgn = sr * sc
                lam_r = sh(lam, sr, ax_r)   # lam at p + sr e_r
                lam_c = sh(lam, sc, ax_c)
                mu_r = sh(mu, sr, ax_r)
                mu_c = sh(mu, sc, ax_c)
                base[..., b, r, c] = sgn * (lam_r + mu_c) / (4 * hr * hc)
                base[..., b, c, r] = sgn * (lam_c + mu_r) / (4 * hr * hc)
    st = -dt * base
    inter = interior_mask(m, n, o, xp, yp, zp)
    fixv = -dt * 2 * ((lam + 2 * mu) / dx / dx + mu / dy / dy + mu / dz / dz)
    out = np.where(inter[..., None, None, None], st, 0.0)
    bnd = ~inter
    out[bnd, 13] = np.eye(3)[None] * fixv[bnd][:, None, None]
    return np.ascontiguousarray(out.reshape(o * n * m, 27, 9))


def random_strain(seed, m, n, o, periodic, std=1e-3):
    """Cell-centred symmetric tensor field, 6 i.i.d. N(0, std) components per
    cell (s11, s12, s13, s22, s23, s33), numpy default_rng(seed) (PCG64).
    Cell counts: N nodes per periodic dim, N-1 cells per Dirichlet dim."""
    xp, yp, zp = periodic
    mc = m if xp else m - 1
    nc = n if yp else n - 1
    oc = o if zp else o - 1
    rng = np.random.default_rng(seed)
    return rng.standard_normal(size=(oc, nc, mc, 6)) * std


def rhs_divergence(eps, m, n, o, periodic, dx, dy, dz):
    """Node divergence of a cell-centred tensor field, the r_field of the
    reference (src/shear_sim_3d.hh:283-385, default sim case with the plates
    at rest) using the 8-cell averaged differences of
    calculate_first_order_stresses (src/shear_sim_3d.cpp:979-998), evaluated
    in the same order.  Non-interior (Dirichlet) nodes get 0.
    Returns (npts, 3)."""
    xp, yp, zp = periodic
    oc, nc, mc, _ = eps.shape
    # pad cells so that cell index -1 is valid: periodic wrap or a dummy layer
    def cell(c, di, dj, dk):
        # value of component c at cell (i+di, j+dj, k+dk) for every node (i,j,k)
        a = eps[..., c]
        ks = (np.arange(o) + dk)
        js = (np.arange(n) + dj)
        is_ = (np.arange(m) + di)
        ks = ks % oc if zp else np.clip(ks, 0, oc - 1)
        js = js % nc if yp else np.clip(js, 0, nc - 1)
        is_ = is_ % mc if xp else np.clip(is_, 0, mc - 1)
        return a[np.ix_(ks, js, is_)]
    S11, S12, S13, S22, S23, S33 = range(6)
    dxi, dyi, dzi = 1.0 / dx, 1.0 / dy, 1.0 / dz

    def ddx(c):
        s = cell(c, 0, 0, 0) - cell(c, -1, 0, 0)
        s = s + cell(c, 0, -1, 0) - cell(c, -1, -1, 0)
        s = s + cell(c, 0, 0, -1) - cell(c, -1, 0, -1)
        s = s + cell(c, 0, -1, -1) - cell(c, -1, -1, -1)
        return .25 * dxi * s

    def ddy(c):
        s = cell(c, 0, 0, 0) - cell(c, 0, -1, 0)
        s = s + cell(c, -1, 0, 0) - cell(c, -1, -1, 0)
        s = s + cell(c, 0, 0, -1) - cell(c, 0, -1, -1)
        s = s + cell(c, -1, 0, -1) - cell(c, -1, -1, -1)
        return .25 * dyi * s

    def ddz(c):
        s = cell(c, 0, 0, 0) - cell(c, 0, 0, -1)
        s = s + cell(c, -1, 0, 0) - cell(c, -1, 0, -1)
        s = s + cell(c, 0, -1, 0) - cell(c, 0, -1, -1)
        s = s + cell(c, -1, -1, 0) - cell(c, -1, -1, -1)
        return .25 * dzi * s

    dsx = ddx(S11) + ddy(S12) + ddz(S13)
    dsy = ddx(S12) + ddy(S22) + ddz(S23)
    dsz = ddx(S13) + ddy(S23) + ddz(S33)
    r = np.stack([dsx, dsy, dsz], axis=-1)
    inter = interior_mask(m, n, o, xp, yp, zp)
    r[~inter] = 0.0
    return np.ascontiguousarray(r.reshape(o * n * m, 3))


def lognormal_mu(seed, m, n, o, sigma=0.3):
    """Per-node mu = exp(sigma Z), Z ~ N(0,1), numpy default_rng(seed): median 1."""
    rng = np.random.default_rng(seed)
    return np.exp(sigma * rng.standard_normal(size=(o, n, m)))


def grid_spacing(m, n, o, periodic, h=None):
    """dx,dy,dz for a grid: 1/N per dimension unless a uniform h is given
    (N cells = nodes for periodic dims, nodes-1 for Dirichlet dims)."""
    if h is not None:
        return h, h, h
    cells = [m if periodic[0] else m - 1, n if periodic[1] else n - 1, o if periodic[2] else o - 1]
    return tuple(1.0 / c for c in cells)


def stress_update(u, sigma, lam, mu, dt, dx, dy, dz, dims, periodic):
    """The projection-step stress update of the reference
    (src/shear_sim_3d.cpp:681-710) with the velocity derivatives of
    calculate_first_order_velocities (src/shear_sim_3d.cpp:901-916), evaluated
    in the same order: returns (sigma + ds, per-cell sym_mat3::modsq(ds)
    (src/mat3.hh:338-340)).  u: (npts, 3) node velocities in natural order
    (the solution, plates included); sigma: (cells_z, cells_y, cells_x, 6)."""
    m, n, o = dims
    xp, yp, zp = periodic
    oc, nc, mc, _ = sigma.shape
    U = u.reshape(o, n, m, 3)

    def node(c, di, dj, dk):
        ks = (np.arange(oc) + dk) % o
        js = (np.arange(nc) + dj) % n
        is_ = (np.arange(mc) + di) % m
        return U[np.ix_(ks, js, is_)][..., c]

    qx, qy, qz = .25 * (1.0 / dx), .25 * (1.0 / dy), .25 * (1.0 / dz)

    def ddx(c):
        s = node(c, 1, 0, 0) - node(c, 0, 0, 0)
        s = s + node(c, 1, 1, 0) - node(c, 0, 1, 0)
        s = s + node(c, 1, 0, 1) - node(c, 0, 0, 1)
        s = s + node(c, 1, 1, 1) - node(c, 0, 1, 1)
        return qx * s

    def ddy(c):
        s = node(c, 0, 1, 0) - node(c, 0, 0, 0)
        s = s + node(c, 1, 1, 0) - node(c, 1, 0, 0)
        s = s + node(c, 0, 1, 1) - node(c, 0, 0, 1)
        s = s + node(c, 1, 1, 1) - node(c, 1, 0, 1)
        return qy * s

    def ddz(c):
        s = node(c, 0, 0, 1) - node(c, 0, 0, 0)
        s = s + node(c, 1, 0, 1) - node(c, 1, 0, 0)
        s = s + node(c, 0, 1, 1) - node(c, 0, 1, 0)
        s = s + node(c, 1, 1, 1) - node(c, 1, 1, 0)
        return qz * s

    du_dx, du_dy, du_dz = ddx(0), ddy(0), ddz(0)
    dv_dx, dv_dy, dv_dz = ddx(1), ddy(1), ddz(1)
    dw_dx, dw_dy, dw_dz = ddx(2), ddy(2), ddz(2)
    ds11 = dt * (lam * (dw_dz + dv_dy) + (lam + 2 * mu) * du_dx)
    ds12 = dt * mu * (du_dy + dv_dx)
    ds13 = dt * mu * (du_dz + dw_dx)
    ds22 = dt * (lam * (dw_dz + du_dx) + (lam + 2 * mu) * dv_dy)
    ds23 = dt * mu * (dv_dz + dw_dy)
    ds33 = dt * (lam * (dv_dy + du_dx) + (lam + 2 * mu) * dw_dz)
    ds = np.stack([ds11, ds12, ds13, ds22, ds23, ds33], axis=-1)
    modsq = 0.5 * (ds11 * ds11 + ds12 * ds12 + ds13 * ds13 + ds12 * ds12 + ds22 * ds22 + ds23 * ds23
                   + ds13 * ds13 + ds23 * ds23 + ds33 * ds33)
    return sigma + ds, modsq
