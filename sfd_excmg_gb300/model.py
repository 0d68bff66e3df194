"""Model container and the reference's input formats.

``Model`` holds what ``read_input`` (sfd_excmg/src/file_opt.f90:8-95) returns:
mesh spacings (air layers first in ``c``), the conductivity tensor per cell
as Fortran ``sigma(ncell,6)`` (numpy shape ``(6, ncell)``), frequencies and
receivers.  Reading goes through the C ABI (``sfdx_read_model``) so the
Fortran host and Python read the same bytes the same way; writing follows
the layout of the reference's generator (sfd_excmg/input.py:6-121).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import capi


@dataclass
class Model:
    nx: int
    ny: int
    nz: int  # total z cells, air included
    nair: int
    a: np.ndarray
    b: np.ndarray
    c: np.ndarray
    sigma: np.ndarray  # (6, ncell): xx yy zz xy xz yz
    freq: np.ndarray
    recv: np.ndarray  # (nrec, 3)
    level: int = 3
    eps: float = 1e-8
    solver: int = 1
    out_type: int = 1
    abu: np.ndarray = field(default_factory=lambda: np.zeros(6, np.int32))
    topo: np.ndarray | None = None  # optional (n1, n2, heights) written as .topo

    @property
    def ncell(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def nl(self) -> int:
        nx, ny, nz = self.nx, self.ny, self.nz
        return nx * (ny + 1) * (nz + 1) + (nx + 1) * ny * (nz + 1) + (nx + 1) * (ny + 1) * nz

    @property
    def nf(self) -> int:
        return len(self.freq)

    def validate(self) -> None:
        if not (len(self.a) == self.nx and len(self.b) == self.ny and len(self.c) == self.nz):
            raise ValueError(f"spacings ({len(self.a)}, {len(self.b)}, {len(self.c)}) do not match the mesh "
                             f"({self.nx}, {self.ny}, {self.nz})")
        if np.shape(self.sigma) != (6, self.ncell):
            raise ValueError(f"sigma has shape {np.shape(self.sigma)}, expected (6, {self.ncell})")
        if np.ndim(self.recv) != 2 or np.shape(self.recv)[1] != 3:
            raise ValueError(f"receivers have shape {np.shape(self.recv)}, expected (nrec, 3)")

    # ------------------------------------------------------------------ I/O
    @classmethod
    def read(cls, name: str, sigma_air: float | None = None) -> "Model":
        """read_input (+ read_topo when the .fwd asks for it) through the C ABI."""
        L = capi.lib()
        dims = [ctypes.c_int() for _ in range(6)]
        capi.check(L.sfdx_read_sizes(name.encode(), *[ctypes.byref(d) for d in dims]), "sfdx_read_sizes")
        nx, ny, nz, nair, nf, nrec = (d.value for d in dims)
        o = capi.Opts.defaults()
        if sigma_air is not None:
            o.sigma_air = sigma_air
        a, b, c = np.zeros(nx), np.zeros(ny), np.zeros(nz)
        sig = np.zeros((6, nx * ny * nz))
        freq = np.zeros(nf)
        recv = np.zeros((3, nrec))
        abu = np.zeros(6, np.int32)
        lev, slv, ot = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        eps = ctypes.c_double()
        capi.check(L.sfdx_read_model(name.encode(), ctypes.byref(o), ctypes.byref(lev), ctypes.byref(eps),
                                     ctypes.byref(slv), ctypes.byref(ot), capi.dptr(a), capi.dptr(b), capi.dptr(c),
                                     capi.dptr(sig), capi.dptr(freq), capi.dptr(recv), capi.iptr(abu)),
                   "sfdx_read_model")
        return cls(nx, ny, nz, nair, a, b, c, sig, freq, np.ascontiguousarray(recv.T), lev.value, eps.value,
                   slv.value, ot.value, abu)

    def write(self, name: str, conduc_type: int | None = None, title: str = "model written by sfd_excmg_gb300",
              ext=(1.15, 1.08)) -> None:
        """Write <name>.fwd / <name>.dat (and <name>.topo) in the reference's layout."""
        self.validate()
        nze = self.nz - self.nair
        if conduc_type is None:
            off = np.any(self.sigma[3:] != 0)
            iso = np.all(self.sigma[0] == self.sigma[1]) and np.all(self.sigma[0] == self.sigma[2])
            conduc_type = 3 if off else (1 if iso else 2)
        with open(name + ".fwd", "w") as f:
            f.write(title.replace("\n", " ") + "\n")
            f.write("%d %e %d %d\n" % (self.level, self.eps, self.solver, self.out_type))
            f.write("%d %d %d %d %d\n" % (self.nx, self.ny, nze, self.nair, 1 if self.topo is not None else 0))
            f.write(" ".join("%.17e" % v for v in self.a) + "\n")
            f.write(" ".join("%.17e" % v for v in self.b) + "\n")
            f.write(" ".join("%.17e" % v for v in self.c[self.nair:]) + "\n")
            f.write("%f %f\n" % ext)
            f.write(" ".join("%d" % v for v in self.abu) + "\n")
            f.write("%d\n" % conduc_type)
            nxy = self.nx * self.ny
            earth = self.sigma[:, self.nair * nxy:]
            ncols = {1: 1, 2: 3, 3: 6}[conduc_type]
            np.savetxt(f, earth[:ncols].T, fmt="%.17e")
        with open(name + ".dat", "w") as f:
            f.write("%d\n" % self.nf)
            for v in self.freq:
                f.write("%.17e\n" % v)
            f.write("%d\n" % self.recv.shape[0])
            for r in self.recv:
                f.write("%.17e %.17e %.17e\n" % tuple(r))
        if self.topo is not None:
            n1, n2, h = self.topo
            with open(name + ".topo", "w") as f:
                f.write("%d %d\n" % (n1, n2))
                for v in np.asarray(h).ravel():
                    f.write("%.17e\n" % v)


def cell_index(nx, ny, i, j, k):
    """0-based cell index of cell (i, j, k) (0-based)."""
    return (k * ny + j) * nx + i
