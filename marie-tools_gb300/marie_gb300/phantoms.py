"""Bodies, materials, input files and coil placements (host-side set-up).

The reference reads bodies from RHBM .mat files (geo_body_domain.m:5-13) named
in JSON input files (load_inputs.m); load_rhbm and load_inputs read those
formats.  The seeded generators produce the same data (voxel grid, idxS,
epsilon_r, sigma) for the benchmark shapes: a homogeneous sphere and an
ellipsoid phantom with random inner ellipsoids, plus loop-coil placements.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

MU0 = 4e-7 * math.pi
C0 = 299792458.0


def em_constants(freq: float) -> dict:
    """em_constants.m:117-139 with the frequency given directly."""
    e0 = 1.0 / (C0 ** 2 * MU0)
    omega = 2 * math.pi * freq
    lamda = C0 / freq
    return dict(freq=freq, mu0=MU0, c0=C0, e0=e0, omega=omega, k0=2 * math.pi / lamda,
                ce=1j * omega * e0)


@dataclass
class Body:
    n: tuple            # (n1, n2, n3)
    res: float
    origin: np.ndarray  # centre of voxel (0,0,0) [m]
    er: np.ndarray      # (n1,n2,n3) relative permittivity (1 in air)
    se: np.ndarray      # (n1,n2,n3) conductivity [S/m]
    idxS: np.ndarray    # 0-based column-major linear indices of body voxels

    def Mr(self, freq):
        """Mr = er + se/ce (em_assembly.m:14)."""
        ce = em_constants(freq)["ce"]
        return self.er + self.se / ce

    def idx_solution(self, pwl: bool) -> np.ndarray:
        """Component-major idx_solution (geo_body_domain.m:22-34), 0-based."""
        nD = int(np.prod(self.n))
        ql = 12 if pwl else 3
        return np.concatenate([c * nD + self.idxS for c in range(ql)]).astype(np.int64)


def grid_centres(n, res):
    n = np.asarray(n)
    origin = -0.5 * res * (n - 1)
    ax = [origin[d] + res * np.arange(n[d]) for d in range(3)]
    X, Y, Z = np.meshgrid(*ax, indexing="ij")
    return origin, X, Y, Z


def _finish(n, res, origin, er, se, mask):
    idxS = np.nonzero(mask.reshape(-1, order="F"))[0].astype(np.int64)
    er = np.where(mask, er, 1.0)
    se = np.where(mask, se, 0.0)
    return Body(tuple(int(v) for v in n), res, origin, er, se, idxS)


# Gyromagnetic ratio / (2 pi) [Hz/T] of the nuclei MARIE simulates
# (em_constants.m:3-60; physical constants, kept as the reference tabulates them)
GAMMA0 = {"1H": 42.577478518e6, "2H": 6.536e6, "3HE": 32.434e6, "13C": 10.705e6, "15N": -4.316e6,
          "17O": -5.772e6, "23NA": 11.262e6, "25MG": -2.614e6, "31P": 17.235e6, "35CL": 4.171e6,
          "39K": 1.250e6, "59CO": 10.054e6, "79BR": 10.666e6, "87RB": 13.932e6, "129XE": 11.777e6}


def larmor_frequency(B0: float, nucleus: str = "1H") -> float:
    """emc.freq = |gamma0| * B0 (em_constants.m:70)."""
    key = nucleus.upper()
    if key not in GAMMA0:
        raise ValueError(f"unknown nucleus {nucleus!r}")
    return abs(GAMMA0[key]) * float(B0)


def load_inputs(path, bodies_root=None) -> dict:
    """The VIE-relevant fields of a MARIE input file (JSON, load_inputs.m:6-
    60): B0, nucleus and the Larmor frequency, the basis (PWX 1 = PWL), the
    body file (resolved against bodies_root, default <inputs dir>/../bodies),
    and the solver / quadrature settings load_inputs.m fixes (GMRES tol 1e-5,
    HOSVD tol 1e-7, 4 / 8 / 15 points for the far / medium / near zones)."""
    import json
    from pathlib import Path
    path = Path(path)
    d = json.loads(path.read_text())
    root = Path(bodies_root) if bodies_root is not None else path.resolve().parent.parent / "bodies"
    pwx = int(d["Basis_Functions_VIE"])
    out = dict(B0=float(d["B0"]), nucleus=d["Nucleus"], freq=larmor_frequency(d["B0"], d["Nucleus"]),
               PWX=pwx, pwl=pwx == 1, body_file=root / d["BodyFile"] if d.get("BodyFile") else None,
               coil_file=d.get("CoilFile", ""), wire_file=d.get("WireFile", ""), shield_file=d.get("ShieldFile", ""),
               tol=1e-5, tol_HOSVD=1e-7, Np_1D_far_V=4, Np_1D_medium_V=8, Np_1D_near_S=15)
    return out


def load_rhbm(path) -> Body:
    """A body file in MARIE's RHBM format (the reference's
    data/bodies/.../*.mat: struct RHBM with fields r (n1 x n2 x n3 x 3 voxel
    centres), epsilon_r, sigma_e (n1 x n2 x n3) and idxS (1-based body voxel
    indices)), read as geo_body_domain.m:5-14 and em_assembly.m:10-12 read
    it: grid edges from size(r), res = |r(2,1,1,1) - r(1,1,1,1)|, the body
    from idxS (made 0-based), materials as stored.  MATLAB v5 .mat files
    (scipy.io); a v7.3 (HDF5) file raises ValueError."""
    import scipy.io as sio
    try:
        S = sio.loadmat(str(path), squeeze_me=False)
    except NotImplementedError as e:     # v7.3 files
        raise ValueError(f"{path}: MATLAB v7.3 (HDF5) body files are not supported; save with -v7") from e
    if "RHBM" not in S:
        raise ValueError(f"{path}: no RHBM struct")
    R = S["RHBM"][0, 0]
    r = np.asarray(R["r"], dtype=np.float64)
    if r.ndim != 4 or r.shape[3] != 3:
        raise ValueError(f"{path}: RHBM.r has shape {r.shape}, expected n1 x n2 x n3 x 3")
    n = tuple(int(v) for v in r.shape[:3])
    res = abs(r[1, 0, 0, 0] - r[0, 0, 0, 0]) if n[0] > 1 else abs(r[0, 1, 0, 1] - r[0, 0, 0, 1])
    er = np.asarray(R["epsilon_r"], dtype=np.float64).reshape(n)
    se = np.asarray(R["sigma_e"], dtype=np.float64).reshape(n)
    idxS = np.asarray(R["idxS"], dtype=np.int64).reshape(-1) - 1
    if idxS.size and (idxS.min() < 0 or idxS.max() >= int(np.prod(n))):
        raise ValueError(f"{path}: RHBM.idxS outside the {n} grid")
    return Body(n, float(res), r[0, 0, 0, :].copy(), er, se, idxS)


def sphere(n=32, res=5e-3, radius=0.06, er=50.0, se=0.6) -> Body:
    """Homogeneous dielectric sphere centred in an n^3 grid."""
    nn = (n, n, n) if np.isscalar(n) else tuple(n)
    origin, X, Y, Z = grid_centres(nn, res)
    mask = X ** 2 + Y ** 2 + Z ** 2 <= radius ** 2
    return _finish(nn, res, origin, np.full(nn, er), np.full(nn, se), mask)


def ellipsoid_phantom(n=96, res=2e-3, axes=(0.080, 0.065, 0.090), n_inner=12, seed=0,
                      shell_er=50.0, shell_se=0.6, scale=1.0) -> Body:
    """Outer ellipsoid (semi-axes `axes`, scaled) with `n_inner` random inner
    ellipsoids, er ~ U[5,80], sigma ~ U[0.02, 2.0]; later ones overwrite
    earlier ones; air outside (excluded from idxS)."""
    rng = np.random.default_rng(seed)
    nn = (n, n, n) if np.isscalar(n) else tuple(n)
    origin, X, Y, Z = grid_centres(nn, res)
    a = np.asarray(axes) * scale
    outer = (X / a[0]) ** 2 + (Y / a[1]) ** 2 + (Z / a[2]) ** 2 <= 1.0
    er = np.full(nn, shell_er)
    se = np.full(nn, shell_se)
    for _ in range(n_inner):
        # centre uniformly inside the half-size ellipsoid, axes 10-35 % of the outer ones
        while True:
            u = rng.uniform(-1, 1, 3)
            if np.sum(u ** 2) <= 1:
                break
        c = 0.5 * a * u
        ai = a * rng.uniform(0.10, 0.35, 3)
        e_r = rng.uniform(5, 80)
        s_e = rng.uniform(0.02, 2.0)
        m = ((X - c[0]) / ai[0]) ** 2 + ((Y - c[1]) / ai[1]) ** 2 + ((Z - c[2]) / ai[2]) ** 2 <= 1.0
        er = np.where(m, e_r, er)
        se = np.where(m, s_e, se)
    return _finish(nn, res, origin, er, se, outer)


def loop_outside(body_axes, gap=0.01, radius=0.05):
    """One loop facing +x, its plane `gap` outside the phantom surface:
    returns (loops (1,6) = centre xyz + normal xyz, radius)."""
    x = body_axes[0] + gap
    return np.array([[x, 0.0, 0.0, 1.0, 0.0, 0.0]]), radius


def loop_ring(n_loops=64, ring_radius=0.16, z_extent=0.16, jitter_deg=10.0, seed=1, n_angles=8):
    """`n_loops` loops on a cylinder of radius `ring_radius`: a uniform grid
    in angle x z, normals radial with a random tilt of up to `jitter_deg`."""
    rng = np.random.default_rng(seed)
    n_z = n_loops // n_angles
    out = []
    for iz in range(n_z):
        z = -z_extent / 2 + z_extent * (iz + 0.5) / n_z
        for ia in range(n_angles):
            phi = 2 * math.pi * (ia + 0.5 * (iz % 2)) / n_angles
            c = np.array([ring_radius * math.cos(phi), ring_radius * math.sin(phi), z])
            nrm = -c.copy()
            nrm[2] = 0.0
            nrm /= np.linalg.norm(nrm)
            # tilt by up to jitter_deg about a random axis perpendicular to the normal
            t = math.radians(jitter_deg) * rng.uniform(0, 1)
            ax = np.cross(nrm, rng.normal(size=3))
            ax /= np.linalg.norm(ax)
            nrm = nrm * math.cos(t) + np.cross(ax, nrm) * math.sin(t) + ax * np.dot(ax, nrm) * (1 - math.cos(t))
            out.append(np.r_[c, nrm])
    return np.array(out)
