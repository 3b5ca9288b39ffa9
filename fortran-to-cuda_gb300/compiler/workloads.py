"""Seeded synthetic workloads of the advection driver (inputs only).

The reference driver fills U, V, W with gfortran's ``random_number`` under a
fixed seed (benchmarks/cdu/src/main.f90:57-64); that generator is not
reproducible outside gfortran, so the restated driver uses the recipe below,
generated on the host with numpy and fed identically to the oracle and the GPU.

Recipe (per velocity, in the order U, V, W): four sine modes
``A*sin(2*pi*(kx*x/Lx + ky*y/Ly + kz*z/Lz) + phi)`` with A = 1 m/s, integer
wavenumbers drawn from 1..4 and phases uniform in [0, 2*pi) (draw order per mode:
kx, ky, kz, phi), evaluated at the field's Arakawa-C position (U on east faces,
V on north faces, W on top faces), plus N(0, 0.05) noise over the interior in
Fortran element order. Then scalars: uniform[280, 300], uniform[0, 0.02], a
Gaussian blob (no draws), then further blobs. Boundaries: periodic x and y;
W zero on the bottom and top wall faces with sign-changed mirrors, the other
fields mirrored (the fill of ``f2c_halo_fill_v1``).

Arrays are numpy float64 of shape (nz+2h, ny+2h, nx+2h), C order == Fortran
column-major (nx+2h, ny+2h, nz+2h).
"""

from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass(frozen=True)
class Geometry:
    nx: int
    ny: int
    nz: int
    halo: int = 2
    dx: float = 10.0
    dy: float = 10.0
    dz: float = 5.0

    @property
    def shape(self):
        h = self.halo
        return (self.nz + 2 * h, self.ny + 2 * h, self.nx + 2 * h)

    @property
    def points(self) -> int:
        return self.nx * self.ny * self.nz

    @property
    def field_bytes(self) -> int:
        return int(np.prod(self.shape)) * 8

    def interior(self):
        h = self.halo
        return (slice(h, h + self.nz), slice(h, h + self.ny), slice(h, h + self.nx))


@dataclass
class Fields:
    geometry: Geometry
    U: np.ndarray
    V: np.ndarray
    W: np.ndarray
    scalars: list = field(default_factory=list)

    def arrays(self):
        return [self.U, self.V, self.W, *self.scalars]


def fill_halo(f: np.ndarray, kind: int, h: int) -> np.ndarray:
    """Host-side boundary fill with the semantics of ``f2c_halo_fill_v1`` (input preparation)."""
    nz, ny, nx = (s - 2 * h for s in f.shape)
    f[h:h + nz, h:h + ny, h + nx:] = f[h:h + nz, h:h + ny, h:2 * h]
    f[h:h + nz, h:h + ny, :h] = f[h:h + nz, h:h + ny, nx:nx + h]
    f[h:h + nz, h + ny:, :] = f[h:h + nz, h:2 * h, :]
    f[h:h + nz, :h, :] = f[h:h + nz, ny:ny + h, :]
    for g in range(h):
        if kind == 0:
            f[h - 1 - g] = f[h + g]
            f[h + nz + g] = f[h + nz - 1 - g]
        else:
            if g == 0:
                f[h - 1] = 0.0
                f[h + nz - 1] = 0.0
            else:
                f[h - 1 - g] = -f[h - 1 + g]
            f[h + nz + g] = -f[h + nz - 2 - g]
    return f


def _coordinates(geo: Geometry, stagger):
    h = geo.halo
    sx, sy, sz = stagger
    x = (np.arange(geo.nx + 2 * h) - h + (1.0 if sx else 0.5)) * geo.dx
    y = (np.arange(geo.ny + 2 * h) - h + (1.0 if sy else 0.5)) * geo.dy
    z = (np.arange(geo.nz + 2 * h) - h + (1.0 if sz else 0.5)) * geo.dz
    return x, y, z


def sine_modes(rng: np.random.Generator, geo: Geometry, stagger, modes: int = 4, amplitude: float = 1.0,
               noise: float = 0.05) -> np.ndarray:
    x, y, z = _coordinates(geo, stagger)
    lx, ly, lz = geo.nx * geo.dx, geo.ny * geo.dy, geo.nz * geo.dz
    out = np.zeros(geo.shape)
    for _ in range(modes):
        kx, ky, kz = (int(v) for v in rng.integers(1, 5, size=3))
        phi = float(rng.uniform(0.0, 2.0 * math.pi))
        phase = (2.0 * math.pi * kz / lz) * z[:, None, None] + (2.0 * math.pi * ky / ly) * y[None, :, None] \
            + ((2.0 * math.pi * kx / lx) * x[None, None, :] + phi)
        out += amplitude * np.sin(phase)
    if noise:
        out[geo.interior()] += rng.normal(0.0, noise, size=(geo.nz, geo.ny, geo.nx))
    return out


def blob(geo: Geometry, centre=(0.5, 0.5, 0.5), width: float = 0.125) -> np.ndarray:
    x, y, z = _coordinates(geo, (False, False, False))
    lx, ly, lz = geo.nx * geo.dx, geo.ny * geo.dy, geo.nz * geo.dz
    sigma = width * min(lx, ly, lz)
    r2 = ((z[:, None, None] - centre[2] * lz) ** 2 + (y[None, :, None] - centre[1] * ly) ** 2
          + (x[None, None, :] - centre[0] * lx) ** 2)
    return np.exp(-r2 / (2.0 * sigma * sigma))


def advection_fields(geo: Geometry, seed: int, nscalar: int = 0) -> Fields:
    """The BASELINE sine-mode velocities plus ``nscalar`` passive scalars, boundaries filled."""
    rng = np.random.default_rng(seed)
    h = geo.halo
    U = fill_halo(sine_modes(rng, geo, (True, False, False)), 0, h)
    V = fill_halo(sine_modes(rng, geo, (False, True, False)), 0, h)
    W = fill_halo(sine_modes(rng, geo, (False, False, True)), 1, h)
    scalars = []
    for n in range(nscalar):
        s = np.zeros(geo.shape)
        if n == 0:
            s[geo.interior()] = rng.uniform(280.0, 300.0, size=(geo.nz, geo.ny, geo.nx))
        elif n == 1:
            s[geo.interior()] = rng.uniform(0.0, 0.02, size=(geo.nz, geo.ny, geo.nx))
        else:
            s = blob(geo, centre=(0.5, 0.5, 0.25 + 0.25 * (n - 2)))
        scalars.append(fill_halo(s, 0, h))
    return Fields(geo, U, V, W, scalars)


def reference_driver_fields(nx: int, ny: int, nz: int, seed: int) -> Fields:
    """The reference driver's geometry (one ghost layer, dx = 1/N, main.f90:47-55) with uniform[0,1) values.

    gfortran's generator is replaced by numpy's; every value, ghosts included, is drawn, as
    ``random_number`` fills the whole arrays there.
    """
    geo = Geometry(nx, ny, nz, halo=1, dx=1.0 / nx, dy=1.0 / ny, dz=1.0 / nz)
    rng = np.random.default_rng(seed)
    U, V, W = (rng.random(geo.shape) for _ in range(3))
    return Fields(geo, U, V, W, [])


# --- batched ensemble and serving samplers ------------------------------------------------------

ENSEMBLE_XY = (64, 96, 128, 192, 256)
ENSEMBLE_Z = (32, 64, 96)


def ensemble_shapes(count: int = 64, seed: int = 1):
    """(nx, ny, nz) per instance: nx, ny uniform over {64..256}, nz over {32,64,96}; draw order nx, ny, nz."""
    rng = np.random.default_rng(seed)
    shapes = []
    for _ in range(count):
        nx = ENSEMBLE_XY[int(rng.integers(0, len(ENSEMBLE_XY)))]
        ny = ENSEMBLE_XY[int(rng.integers(0, len(ENSEMBLE_XY)))]
        nz = ENSEMBLE_Z[int(rng.integers(0, len(ENSEMBLE_Z)))]
        shapes.append((nx, ny, nz))
    return shapes


def advection_fields_device(geo: Geometry, seed: int, nscalar: int, torch, device="cuda"):
    """The sine-mode recipe generated on the GPU with torch's generator (fast; not bit-equal to the numpy draw).

    Used by the benchmark's large ensembles; parity tests use ``advection_fields``.
    Returns a list of device tensors U, V, W, S1.. of shape ``geo.shape``.
    """
    g = torch.Generator(device=device)
    g.manual_seed(seed)
    h = geo.halo
    lx, ly, lz = geo.nx * geo.dx, geo.ny * geo.dy, geo.nz * geo.dz
    out = []
    for stagger in ((True, False, False), (False, True, False), (False, False, True)):
        x, y, z = (torch.as_tensor(c, device=device) for c in _coordinates(geo, stagger))
        field = torch.zeros(geo.shape, dtype=torch.float64, device=device)
        for _ in range(4):
            k = torch.randint(1, 5, (3,), generator=g, device=device).tolist()
            phi = float(torch.rand((), generator=g, device=device, dtype=torch.float64)) * 2.0 * math.pi
            field += torch.sin((2.0 * math.pi * k[2] / lz) * z[:, None, None] + (2.0 * math.pi * k[1] / ly) *
                               y[None, :, None] + ((2.0 * math.pi * k[0] / lx) * x[None, None, :] + phi))
        inner = field[h:h + geo.nz, h:h + geo.ny, h:h + geo.nx]
        inner += 0.05 * torch.randn(inner.shape, generator=g, device=device, dtype=torch.float64)
        out.append(field)
    for n in range(nscalar):
        s = torch.zeros(geo.shape, dtype=torch.float64, device=device)
        inner = s[h:h + geo.nz, h:h + geo.ny, h:h + geo.nx]
        if n == 0:
            inner.copy_(280.0 + 20.0 * torch.rand(inner.shape, generator=g, device=device, dtype=torch.float64))
        elif n == 1:
            inner.copy_(0.02 * torch.rand(inner.shape, generator=g, device=device, dtype=torch.float64))
        else:
            s.copy_(torch.as_tensor(blob(geo, centre=(0.5, 0.5, 0.25 + 0.25 * (n - 2))), device=device))
        out.append(s)
    return out


# --- host statement of the device job generator (f2c_seed_fields_v1) -------------------------------

_MASK = (1 << 64) - 1
_GOLDEN = 0x9E3779B97F4A7C15


def _mix64_int(z: int) -> int:
    z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _MASK
    z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _MASK
    return z ^ (z >> 31)


def _mix64(z: np.ndarray) -> np.ndarray:
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def _uniform(key: int, n: np.ndarray) -> np.ndarray:
    z = np.uint64(key) + np.uint64(_GOLDEN) * (n + np.uint64(1))
    return (_mix64(z) >> np.uint64(11)).astype(np.float64) * 2.0 ** -53


def _uniform24(key: int, n: np.ndarray) -> np.ndarray:
    z = np.uint64(key) + np.uint64(_GOLDEN) * (n + np.uint64(1))
    return (_mix64(z) >> np.uint64(40)).astype(np.float32) * np.float32(2.0 ** -24)


def seeded_fields_reference(geo: Geometry, seed: int, nscalar: int = 0) -> list:
    """The fields ``f2c_seed_fields_v1`` writes on the device, computed on the host with numpy.

    Per velocity four sine modes (wavenumbers 1..4 per axis and a phase, drawn on the host from a splitmix64
    stream of the seed) at the staggered position, plus N(0, 0.05) noise from counter-based draws of the point's
    interior index (Box-Muller), evaluated in single precision in the device's order of operations; scalar 0
    uniform in [280, 300] and scalar 1 in [0, 0.02] (53-bit draws), further scalars Gaussian blobs (single
    precision); ghosts filled by the boundary rule. Agrees with the device to the rounding of the single-precision
    sin, cos, log and exp (a few units in the last place of a float).
    """
    f32 = np.float32
    with np.errstate(over="ignore"):
        state = _mix64_int(seed ^ 0x5EEDF1E1D5)

        def draw() -> int:
            nonlocal state
            state = (state + _GOLDEN) & _MASK
            return _mix64_int(state)

        lengths = (geo.nx * geo.dx, geo.ny * geo.dy, geo.nz * geo.dz)
        modes = []
        for _ in range(3):
            per = []
            for _ in range(4):
                k = [1.0 + float(draw() % 4) for _ in range(3)]
                phi = 2.0 * math.pi * (float(draw() >> 11) * 2.0 ** -53)
                per.append([f32(2.0 * math.pi * k[a] / lengths[a]) for a in range(3)] + [f32(phi)])
            modes.append(per)
        keys = [draw() for _ in range(7)]
        k, j, i = np.meshgrid(np.arange(geo.nz), np.arange(geo.ny), np.arange(geo.nx), indexing="ij")
        n = (i + geo.nx * (j + geo.ny * k)).astype(np.uint64)
        fi, fj, fk = i.astype(f32), j.astype(f32), k.astype(f32)
        dx, dy, dz = f32(geo.dx), f32(geo.dy), f32(geo.dz)
        out = []
        for c in range(3):
            x = (fi + f32(1.0 if c == 0 else 0.5)) * dx
            y = (fj + f32(1.0 if c == 1 else 0.5)) * dy
            z = (fk + f32(1.0 if c == 2 else 0.5)) * dz
            v = np.zeros(n.shape, dtype=f32)
            for ax, ay, az, phi in modes[c]:
                v = v + np.sin(az * z + ay * y + (ax * x + phi))
            u1 = f32(1.0) - _uniform24(keys[c], np.uint64(2) * n)
            u2 = _uniform24(keys[c], np.uint64(2) * n + np.uint64(1))
            v = v + f32(0.05) * (np.sqrt(f32(-2.0) * np.log(u1)) * np.cos(f32(6.28318530717958648) * u2))
            out.append(v.astype(np.float64))
        lx, ly, lz = (f32(geo.nx) * dx, f32(geo.ny) * dy, f32(geo.nz) * dz)
        sigma = f32(0.125) * min(lx, ly, lz)
        for s in range(nscalar):
            if s == 0:
                v = 280.0 + 20.0 * _uniform(keys[3], n)
            elif s == 1:
                v = 0.02 * _uniform(keys[4], n)
            else:
                x = (fi + f32(0.5)) * dx - f32(0.5) * lx
                y = (fj + f32(0.5)) * dy - f32(0.5) * ly
                z = (fk + f32(0.5)) * dz - f32(0.25 + 0.25 * (s - 2)) * lz
                v = np.exp(-(x * x + y * y + z * z) / (f32(2.0) * sigma * sigma)).astype(np.float64)
            out.append(v)
    fields = []
    for c, v in enumerate(out):
        f = np.zeros(geo.shape)
        f[geo.interior()] = v
        fields.append(fill_halo(f, 1 if c == 2 else 0, geo.halo))
    return fields
