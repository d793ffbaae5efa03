"""Deterministic synthetic Lyman-alpha skewer data in Dachshund's formats.

There is no public dataset for this path: the inputs are seeded synthetic
skewers with the shapes of the workloads this library is measured on.  Every
generator returns ``Pixel`` records as an ``(n, 5)`` float64 array
``{x, y, z, n, d}`` (the reference's binary pixel format, lib/pixel.h:16-22,
README.md:32-36), skewer-contiguous, plus the matching run parameters.

Kernel parameters shared by all workloads: var_s = sigma_F^2 = 0.0625,
l_perp = 2.5 Mpc/h, l_para = 2.0 Mpc/h.  Pixels sit at z_k = (k + 0.5) dz with
dz = 2 Mpc/h; noise n ~ U[0.05, 0.3].

Data d:
* ``dense``: d ~ N(0, S + diag(n^2)) drawn by a dense Cholesky factor of the
  exact-exp covariance (small problems only);
* ``grf``: a Gaussian random field with the kernel's own power spectrum
  P(k) = var_s (2 pi)^{3/2} l_perp^2 l_para exp(-(k_perp^2 l_perp^2 +
  k_para^2 l_para^2)/2), drawn by FFT on a periodic 1 Mpc/h grid, trilinearly
  interpolated to the pixels, plus n * N(0, 1).
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

VAR_S = 0.0625
L_PERP = 2.5
L_PARA = 2.0
DZ = 2.0


@dataclasses.dataclass
class Workload:
    """One solve: pixels plus the reference app's run parameters."""

    name: str
    pixels: np.ndarray          # (n, 5) Pixel records {x, y, z, n, d}
    lx: float
    ly: float
    lz: float
    map_nx: int
    map_ny: int
    map_nz: int
    var_s: float = VAR_S
    l_perp: float = L_PERP
    l_para: float = L_PARA
    pcg_tol: float = 1e-8
    pcg_max_iter: int = 1000
    pcg_step_r: int = 50
    n_skewers: int = 0
    pix_per_skewer: int = 0

    @property
    def n(self) -> int:
        return int(self.pixels.shape[0])

    @property
    def n_map(self) -> int:
        return self.map_nx * self.map_ny * self.map_nz

    def config_text(self, pixel_path: str = "pixels.bin", map_path: str = "map.bin") -> str:
        """The reference app's ``key = value`` config (app/dachshund.cc:62-159)."""
        kv = [
            ("lx", repr(self.lx)), ("ly", repr(self.ly)), ("lz", repr(self.lz)),
            ("num_pixels", str(self.n)),
            ("map_nx", str(self.map_nx)), ("map_ny", str(self.map_ny)),
            ("map_nz", str(self.map_nz)),
            ("corr_var_s", repr(self.var_s)), ("corr_l_perp", repr(self.l_perp)),
            ("corr_l_para", repr(self.l_para)),
            ("pcg_tol", repr(self.pcg_tol)), ("pcg_max_iter", str(self.pcg_max_iter)),
            ("pcg_step_r", str(self.pcg_step_r)),
            ("pixel_data_path", pixel_path), ("map_path", map_path),
        ]
        return "".join(f"{k} = {v}\n" for k, v in kv)

    def write(self, directory: str) -> str:
        """Write ``pixels.bin`` + ``run.cfg``; returns the config path."""
        os.makedirs(directory, exist_ok=True)
        directory = os.path.abspath(directory)
        pix_path = os.path.join(directory, "pixels.bin")
        np.ascontiguousarray(self.pixels, dtype=np.float64).tofile(pix_path)
        cfg = os.path.join(directory, "run.cfg")
        with open(cfg, "w") as f:
            f.write(self.config_text(pix_path, os.path.join(directory, "map.bin")))
        return cfg


def skewer_pixels(rng, n_sk, n_per, box_xy, dz=DZ, noise=(0.05, 0.3)):
    """Skewers at uniform (x, y) in [0, box_xy)^2, pixels at z_k = (k+1/2) dz."""
    xy = rng.uniform(0.0, box_xy, size=(n_sk, 2))
    z = (np.arange(n_per) + 0.5) * dz
    pix = np.empty((n_sk * n_per, 5))
    pix[:, 0] = np.repeat(xy[:, 0], n_per)
    pix[:, 1] = np.repeat(xy[:, 1], n_per)
    pix[:, 2] = np.tile(z, n_sk)
    pix[:, 3] = rng.uniform(noise[0], noise[1], size=n_sk * n_per)
    pix[:, 4] = 0.0
    return pix


def exact_covariance(pts, var_s=VAR_S, l_perp=L_PERP, l_para=L_PARA):
    """Dense exact-exp S (n x n) for small point sets."""
    x, y, z = (np.ascontiguousarray(pts[:, k]) for k in range(3))
    arg = np.subtract.outer(x, x)
    arg *= arg
    t = np.subtract.outer(y, y)
    t *= t
    arg += t
    arg *= 1.0 / (2 * l_perp**2)
    t = np.subtract.outer(z, z)
    t *= t
    t *= 1.0 / (2 * l_para**2)
    arg += t
    np.negative(arg, out=arg)
    np.exp(arg, out=arg)
    arg *= var_s
    return arg


def dense_data(rng, pix, var_s=VAR_S, l_perp=L_PERP, l_para=L_PARA):
    """d ~ N(0, S + diag(n^2)) by dense Cholesky."""
    C = exact_covariance(pix[:, :3], var_s, l_perp, l_para)
    C[np.diag_indices_from(C)] += pix[:, 3] ** 2
    L = np.linalg.cholesky(C)
    return L @ rng.standard_normal(pix.shape[0])


def grf_field(rng, shape, cell=1.0, var_s=VAR_S, l_perp=L_PERP, l_para=L_PARA):
    """Periodic GRF on a grid of ``shape`` cells of side ``cell`` (axes x, y, z)."""
    nx, ny, nz = shape
    kx = 2 * np.pi * np.fft.fftfreq(nx, d=cell)
    ky = 2 * np.pi * np.fft.fftfreq(ny, d=cell)
    kz = 2 * np.pi * np.fft.rfftfreq(nz, d=cell)
    kperp2 = kx[:, None, None] ** 2 + ky[None, :, None] ** 2
    kpara2 = kz[None, None, :] ** 2
    P = var_s * (2 * np.pi) ** 1.5 * l_perp**2 * l_para * np.exp(
        -(kperp2 * l_perp**2 + kpara2 * l_para**2) / 2.0)
    white = rng.standard_normal((nx, ny, nz))
    fk = np.fft.rfftn(white) * np.sqrt(P / cell**3)
    return np.fft.irfftn(fk, s=(nx, ny, nz), axes=(0, 1, 2))


def trilinear(field, pts, cell=1.0):
    """Periodic trilinear interpolation of a cell-centred grid field."""
    nx, ny, nz = field.shape
    g = pts / cell - 0.5
    i0 = np.floor(g).astype(np.int64)
    f = g - i0
    out = np.zeros(pts.shape[0])
    for dx in (0, 1):
        wx = f[:, 0] if dx else 1 - f[:, 0]
        ix = (i0[:, 0] + dx) % nx
        for dy in (0, 1):
            wy = f[:, 1] if dy else 1 - f[:, 1]
            iy = (i0[:, 1] + dy) % ny
            for dz in (0, 1):
                wz = f[:, 2] if dz else 1 - f[:, 2]
                iz = (i0[:, 2] + dz) % nz
                out += wx * wy * wz * field[ix, iy, iz]
    return out


def grf_data(rng, pix, box, cell=1.0, var_s=VAR_S, l_perp=L_PERP, l_para=L_PARA):
    shape = tuple(int(round(b / cell)) for b in box)
    field = grf_field(rng, shape, cell, var_s, l_perp, l_para)
    return trilinear(field, pix[:, :3], cell) + pix[:, 3] * rng.standard_normal(pix.shape[0])


def grf_workload(name, n_sk, n_per, box_xy, seed, map_shape, tol):
    """n_sk skewers of n_per pixels at uniform (x, y) in [0, box_xy)^2 with
    GRF + noise data; map grid ``map_shape`` over the box."""
    rng = np.random.default_rng(seed)
    pix = skewer_pixels(rng, n_sk, n_per, box_xy)
    lz = n_per * DZ
    pix[:, 4] = grf_data(rng, pix, (box_xy, box_xy, lz))
    return Workload(name, pix, float(box_xy), float(box_xy), float(lz), *map_shape,
                    pcg_tol=tol, n_skewers=n_sk, pix_per_skewer=n_per)


def wf4096(seed: int = 0) -> Workload:
    """4,096 pixels: 64 skewers x 64 in [0,32)^2 x [0,128); dense-Cholesky d;
    tol 1e-5, max 200 iterations; map 32 x 32 x 128."""
    rng = np.random.default_rng(seed)
    pix = skewer_pixels(rng, 64, 64, 32.0)
    pix[:, 4] = dense_data(rng, pix)
    return Workload("wf-4096px-dense-d", pix, 32.0, 32.0, 128.0, 32, 32, 128,
                    pcg_tol=1e-5, pcg_max_iter=200, n_skewers=64, pix_per_skewer=64)


def wf32768(seed: int = 0) -> Workload:
    """32,768 pixels: 256 skewers x 128 in [0,40)^2 x [0,256); GRF d; tol 1e-8;
    map 40 x 40 x 256."""
    return grf_workload("wf-32768px-grf", 256, 128, 40.0, seed, (40, 40, 256), 1e-8)


def wf262144(seed: int = 0) -> Workload:
    """262,144 pixels: 1,024 skewers x 256 in [0,80)^2 x [0,512); GRF d;
    tol 1e-8; map 80 x 80 x 512."""
    return grf_workload("wf-262144px-grf", 1024, 256, 80.0, seed, (80, 80, 512), 1e-8)


def small(n_sk=16, n_per=32, box_xy=12.0, seed=0, tol=1e-8) -> Workload:
    """A scaled-down GRF workload for parity tests."""
    lz = n_per * DZ
    return grf_workload(f"wf-{n_sk * n_per}px-small", n_sk, n_per, box_xy, seed,
                         (max(1, int(box_xy)), max(1, int(box_xy)), int(lz)), tol)


def chunks(n_chunks=512, seed=0, sk_range=(16, 192), per_range=(64, 128), spacing=2.5,
           n_rhs=0):
    """Independent sub-volume chunks of uneven size (batched workload).

    Each chunk has a uniform-integer number of skewers and of pixels per skewer;
    its box side is spacing * sqrt(n_skewers), so the mean skewer spacing is
    ``spacing`` Mpc/h; z_k = (k + 1/2) 2 Mpc/h.  d = GRF signal (1 Mpc/h grid,
    trilinear) + n N(0, 1).  Returns a list of (n, 5) Pixel arrays; with
    ``n_rhs`` > 0 also an (n_total, n_rhs) array of data vectors: the same
    signal plus n_rhs independent noise realisations (column 0 is the d of
    the records)."""
    rng = np.random.default_rng(seed)
    out, rhs = [], []
    for _ in range(n_chunks):
        n_sk = int(rng.integers(sk_range[0], sk_range[1] + 1))
        n_per = int(rng.integers(per_range[0], per_range[1] + 1))
        side = spacing * np.sqrt(n_sk)
        pix = skewer_pixels(rng, n_sk, n_per, side)
        shape = (max(2, int(np.ceil(side))), max(2, int(np.ceil(side))), n_per * int(DZ))
        signal = trilinear(grf_field(rng, shape, 1.0), pix[:, :3], 1.0)
        pix[:, 4] = signal + pix[:, 3] * rng.standard_normal(len(pix))
        if n_rhs > 0:
            r = signal[:, None] + pix[:, 3:4] * rng.standard_normal((len(pix), n_rhs))
            r[:, 0] = pix[:, 4]
            rhs.append(r)
        out.append(pix)
    if n_rhs > 0:
        return out, np.ascontiguousarray(np.concatenate(rhs, axis=0))
    return out


def uniform_map_coords(lx, ly, lz, nx, ny, nz) -> np.ndarray:
    """Cell-centred grid, flat index (ix*ny + iy)*nz + iz (lib/util.cc:25-46)."""
    dx, dy, dz = lx / nx, ly / ny, lz / nz
    ix, iy, iz = np.meshgrid(np.arange(nx), np.arange(ny), np.arange(nz), indexing="ij")
    out = np.empty((nx * ny * nz, 3))
    out[:, 0] = (dx * (ix + 0.5)).ravel()
    out[:, 1] = (dy * (iy + 0.5)).ravel()
    out[:, 2] = (dz * (iz + 0.5)).ravel()
    return out


WORKLOADS = {"wf4096": wf4096, "wf32768": wf32768, "wf262144": wf262144}
