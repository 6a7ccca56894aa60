"""Z-slab decomposition of the multigrid's fine level over several GPUs.

The reference splits its grid over MPI ranks (mg_3d_template/geometry.cc)
and keeps every rank's ghost layers current by exchanges: before each
Gauss-Seidel sweep (region::communicate, region.cc:2759-2847), around
restriction and interpolation (the strip exchanges of region.cc:2851-2910),
and it gathers the coarse levels onto fewer ranks (multigrid.cc:47-103).
This module is that decomposition for this library's 8-colour smoother:

* the z-planes are split into contiguous slabs, one per sub-domain; a slab
  is an ordinary handle over its planes plus one ghost plane below and above
  (planes the neighbour owns), laid out so that local and global plane
  parities agree (a spare plane below the ghost where needed);
* colours 0-3 update even planes and read only the odd planes above and
  below, colours 4-7 the reverse, so a sweep needs two one-plane exchanges:
  the odd ghost planes (below each slab) before colour 0 and the even ones
  (above) before colour 4.  Every slab then sees exactly the values the
  undivided colour order gives it: the decomposed sweep is bit-identical;
* the residual norm is a sum over owned planes, all-reduced in FP64;
* restriction needs the residual of the plane below a slab, which is
  exchanged; each slab restricts the coarse planes centred on its own even
  planes, those are gathered onto the root, which runs the coarse levels
  (any solver of the coarse grid) and broadcasts the coarse correction, and
  every slab interpolates it into its own planes.

Transports: :class:`LocalTransport` (all slabs in one process: copies; one
GPU or the CPU) and :class:`DistTransport` (one slab per rank of a
``torch.distributed`` group: point-to-point sends into the receiver's own
buffer, gather to the root, broadcast, all-reduce -- NCCL between GPUs, gloo
on the CPU).  Planes move as ordinary buffers: no TMA, multicast or peer
mapping.  A slab is any object with the methods of :class:`HandleSlab` (the
GPU one, over the C-ABI); the CPU tests supply a numpy one.
"""
from __future__ import annotations

import numpy as np


def partition(o, zp, parts):
    """Owned plane ranges [k0, k1) of `parts` slabs of a level with o planes:
    contiguous, every interior boundary even, as equal as that allows, at
    least 4 planes each (two slabs at least when z is periodic)."""
    if parts < 1 or o < 4 * parts:
        raise ValueError(f"{parts} slabs of {o} planes: at least 4 planes per slab")
    if zp and (o % 2 or parts < 2):
        raise ValueError("a periodic z needs an even number of planes and two slabs at least")
    bounds = [0] + [(p * o // parts) & ~1 for p in range(1, parts)] + [o]
    if any(b <= a for a, b in zip(bounds, bounds[1:])):
        raise ValueError("slabs too thin for even boundaries")
    return [(bounds[p], bounds[p + 1]) for p in range(parts)]


class SlabLayout:
    """Planes of one slab: owned [k0, k1); a ghost below (k0 - 1) and above
    (k1), wrapped when z is periodic, where the grid goes on; stored planes
    start at the even global plane `first` and local plane i is global plane
    first + i (mod o when z is periodic)."""

    def __init__(self, o, zp, k0, k1):
        self.o, self.zp, self.k0, self.k1 = o, zp, k0, k1
        self.lo = zp or k0 > 0
        self.hi = zp or k1 < o
        first = k0 - (1 if self.lo else 0)
        self.first = first - (first & 1)
        self.nplanes = k1 + (1 if self.hi else 0) - self.first

    def local(self, k):
        """Local index of global plane k (owned or ghost)."""
        return (k - self.first) % self.o if self.zp else k - self.first

    def coarse_owned(self):
        """Global coarse planes [K0, K1) this slab restricts: those centred on
        its own even planes, and at the top of a z that is not periodic the
        last coarse plane (which an even number of planes puts on the last,
        odd, fine plane: region.cc:856)."""
        K1 = coarse_planes(self.o, self.zp) if (self.k1 == self.o and not self.zp) else (self.k1 + 1) // 2
        return (self.k0 + 1) // 2, K1

    def coarse_global(self, i, oc):
        """Global coarse plane of local coarse plane i."""
        k = self.first // 2 + i
        return k % oc if self.zp else k


def coarse_planes(o, zp):
    """Planes of the coarse level of a level with o planes (region.cc:856)."""
    return (o + (1 if zp else 2)) >> 1


class LocalTransport:
    """All slabs in this process: planes move by copy."""

    def __init__(self, nslabs):
        self.nslabs = nslabs

    def mine(self):
        return list(range(self.nslabs))

    def exchange(self, sends, recv_like):
        """sends: {p: (q, buf)} -> {q: buf}."""
        return {q: buf for p, (q, buf) in sends.items()}

    def gather(self, parts, like):
        return [parts[p] for p in range(self.nslabs)]

    def bcast(self, buf, like):
        return buf

    def allreduce_sum(self, parts):
        return float(sum(parts[p] for p in sorted(parts)))

    def is_root(self):
        return True


def _tensor(a):
    import torch
    return a if isinstance(a, torch.Tensor) else torch.from_numpy(np.ascontiguousarray(a))


def _like(t, a):
    return t if not isinstance(a, np.ndarray) else t.numpy()


class DistTransport:
    """One slab per rank of a torch.distributed group (slab p on rank p)."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self.d = dist
        self.group = group
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)

    def mine(self):
        return [self.rank]

    def exchange(self, sends, recv_like):
        """sends: {rank: (dest, buf)}; recv_like: {rank: (src, empty buf)} ->
        {rank: received buf}."""
        reqs, out = [], {}
        for p, (src, like) in recv_like.items():
            t = _tensor(like)
            reqs.append(self.d.irecv(t, src, group=self.group))
            out[p] = (t, like)
        for p, (q, buf) in sends.items():
            reqs.append(self.d.isend(_tensor(buf).contiguous(), q, group=self.group))
        for r in reqs:
            r.wait()
        return {p: _like(t, like) for p, (t, like) in out.items()}

    def gather(self, parts, like):
        """parts: {rank: buf}; like(p): an empty buffer of slab p's part (on
        the root) -> the parts in slab order on the root, None elsewhere."""
        mine = _tensor(parts[self.rank]).contiguous()
        if self.rank != 0:
            self.d.send(mine, 0, group=self.group)
            return None
        out = [parts[0]]
        for p in range(1, self.size):
            b = like(p)
            t = _tensor(b)
            self.d.recv(t, p, group=self.group)
            out.append(_like(t, b))
        return out

    def bcast(self, buf, like):
        b = buf if self.rank == 0 else like()
        t = _tensor(b)
        self.d.broadcast(t, 0, group=self.group)
        return _like(t, b)

    def allreduce_sum(self, parts):
        import torch
        dev = "cuda" if self.d.get_backend(self.group) == "nccl" else "cpu"
        t = torch.tensor([parts[self.rank]], dtype=torch.float64, device=dev)
        self.d.all_reduce(t, group=self.group)
        return float(t.item())

    def is_root(self):
        return self.rank == 0


def _concat(parts):
    if isinstance(parts[0], np.ndarray):
        return np.concatenate(parts, axis=0)
    import torch
    return torch.cat(list(parts), dim=0)


class SlabSolver:
    """The decomposed fine-level operations of a grid with o planes (z
    periodic or not) split into len(layouts) slabs; `slabs` maps each local
    slab index (the transport's mine()) to its slab object."""

    def __init__(self, o, zp, layouts, slabs, transport):
        self.o, self.zp = o, zp
        self.layouts = layouts
        self.slabs = slabs
        self.t = transport
        self.P = len(layouts)
        self.oc = coarse_planes(o, zp)

    @classmethod
    def split(cls, o, zp, parts, make_slab, transport):
        """Partition o planes into `parts` slabs and build this process's
        slabs with make_slab(layout)."""
        layouts = [SlabLayout(o, zp, k0, k1) for k0, k1 in partition(o, zp, parts)]
        return cls(o, zp, layouts, {p: make_slab(layouts[p]) for p in transport.mine()}, transport)

    def _neighbour(self, p, up):
        q = p + 1 if up else p - 1
        if 0 <= q < self.P:
            return q
        return q % self.P if self.zp else None

    def exchange(self, which, level, up):
        """Fill one ghost plane of every slab from its neighbour's owned
        plane: up=True sends each slab's top owned plane into the ghost below
        the next slab up, up=False its bottom owned plane into the ghost above
        the next slab down."""
        sends, recvs = {}, {}
        for p in self.t.mine():
            L, s = self.layouts[p], self.slabs[p]
            q = self._neighbour(p, up)
            if q is not None:
                k = L.k1 - 1 if up else L.k0
                sends[p] = (q, s.get_planes(level, which, L.local(k), 1))
            src = self._neighbour(p, not up)
            if src is not None:
                recvs[p] = (src, s.empty_planes(level, 1))
        got = self.t.exchange(sends, recvs)
        for p, buf in got.items():
            L = self.layouts[p]
            k = (L.k0 - 1) % self.o if up else L.k1 % self.o
            self.slabs[p].set_planes(level, which, L.local(k), buf)

    def sweep(self, count=1):
        """`count` 8-colour sweeps of the fine level, bit-identical to the
        undivided sweep."""
        for _ in range(count):
            self.exchange("x", 0, up=True)     # odd ghosts below, read by colours 0-3
            for p in self.t.mine():
                self.slabs[p].colours(0, 4)
            self.exchange("x", 0, up=False)    # even ghosts above, read by colours 4-7
            for p in self.t.mine():
                self.slabs[p].colours(4, 8)

    def residual(self):
        """r - A x on every owned plane (both x ghosts refreshed first);
        returns the FP64 all-reduced |r - A x|^2 of all slabs."""
        self.exchange("x", 0, up=True)
        self.exchange("x", 0, up=False)
        parts = {}
        for p in self.t.mine():
            L, s = self.layouts[p], self.slabs[p]
            s.residual()
            parts[p] = s.sumsq_planes(0, "res", L.local(L.k0), L.k1 - L.k0)
        return self.t.allreduce_sum(parts)

    def restrict_gather(self):
        """The coarse right-hand side of the whole coarse level (natural
        order) on the root, None elsewhere: residual, the residual plane below
        each slab exchanged, restriction per slab, the coarse planes centred on
        each slab's own planes gathered in slab order."""
        self.residual()
        self.exchange("res", 0, up=True)
        parts = {}
        for p in self.t.mine():
            L, s = self.layouts[p], self.slabs[p]
            s.restrict()
            K0, K1 = L.coarse_owned()
            parts[p] = s.get_planes(1, "r", K0 - L.first // 2, K1 - K0)
        like = lambda p: self.slabs[self.t.mine()[0]].empty_planes(1, self.layouts[p].coarse_owned()[1] -
                                                                   self.layouts[p].coarse_owned()[0])
        out = self.t.gather(parts, like)
        return None if out is None else _concat(out)

    def scatter_interpolate(self, xc):
        """Broadcast the coarse correction xc (the whole coarse level, natural
        order; given on the root) and interpolate it into every slab's owned
        planes: fine x += P xc."""
        mine = self.t.mine()
        xc = self.t.bcast(xc, lambda: self.slabs[mine[0]].empty_planes(1, self.oc))
        for p in mine:
            L, s = self.layouts[p], self.slabs[p]
            per = s.plane_size(1)
            ks = [L.coarse_global(i, self.oc) for i in range(s.nplanes(1))]
            sel = _concat([xc[k * per:(k + 1) * per] for k in ks])
            s.set_planes(1, "x", 0, sel)
            s.interpolate()

    def two_level_cycle(self, v_down, v_up, coarse_solve):
        """Pre-sweeps, restriction gathered onto the root, xc = coarse_solve(rc)
        on the root, interpolation, post-sweeps: the fine level of the
        undivided cycle with its coarse levels on one rank."""
        self.sweep(v_down)
        rc = self.restrict_gather()
        xc = coarse_solve(rc) if self.t.is_root() else None
        self.scatter_interpolate(xc)
        self.sweep(v_up)


class HandleSlab:
    """A slab on the GPU: a Multigrid handle over the slab's planes (x and y
    as the grid, z Dirichlet: its end planes are ghosts or spare planes,
    never updated by the decomposition), FP64 fields, the shared stencil,
    two levels at least."""

    def __init__(self, dims_xy, periodic_xy, layout, stencil, fix, device=0):
        import torch
        from .mg import Multigrid
        m, n = dims_xy
        self.mg = Multigrid((m, n, layout.nplanes), (periodic_xy[0], periodic_xy[1], False), precision="fp64",
                            max_coarse=m * n * layout.nplanes - 1, bottom="gs", device=device)
        self.mg.setup_matrices(stencil=stencil, fix=fix)
        self.device = torch.device("cuda", device)

    def close(self):
        self.mg.close()

    def plane_size(self, level):
        m, n, _ = self.mg.level_dims(level)
        return m * n

    def nplanes(self, level):
        return self.mg.level_dims(level)[2]

    def empty_planes(self, level, nk):
        import torch
        return torch.empty((nk * self.plane_size(level), 3), dtype=torch.float64, device=self.device)

    def get_planes(self, level, which, k0, nk):
        return self.mg.level_get_planes(level, which, k0, nk, self.empty_planes(level, nk))

    def set_planes(self, level, which, k0, v):
        self.mg.level_set_planes(level, which, k0, v.contiguous())

    def colours(self, q0, q1):
        self.mg.gauss_seidel_colours(0, q0, q1)

    def residual(self):
        self.mg.compute_residual(0)

    def sumsq_planes(self, level, which, k0, nk):
        v = self.get_planes(level, which, k0, nk)
        return float((v * v).sum())

    def restrict(self):
        self.mg.restrict_residual(1)

    def interpolate(self):
        self.mg.interpolation(1)
