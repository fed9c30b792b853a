"""The benchmark problems: seeded synthetic phantoms, media and beams.

  water30      30^3 x 1 cm water, 2 MeV photon pencil beam along +z,
               ECUT 0.7 MeV, PCUT 0.01 MeV (1e7 histories, 10 batches, seed 1)
  slab64       64^3 x 0.25 cm; z-slabs water 0-3, lung 3-9, ICRP bone 9-11,
               water 11-16 cm; 10x10 cm parallel photon field with energies
               from dN/dE ~ E^-1 (1 - E/6) on 0.1-6 MeV in 1000 histogram bins
               (1e8 histories, seed 2)
  water128e    128^3 x 0.2 cm water, 20 MeV electron 10x10 cm field,
               ECUT 0.521 MeV (2e8 histories, seed 3)
  perturbed64  64^3 x 0.3 cm water with relative densities 1 + 0.1 u,
               u ~ U(-1,1) (seed 11), 6 MeV photon 5x5 cm field (seed 13)
  batched64    64 independent problems run together: cubes of n ~ U{32..160}
               voxels of 0.2 cm whose densities are a Gaussian random field
               (1 cm smoothing) mapped to 0.2-1.9 g/cc and to four media by
               threshold; per problem a photon or electron 10 cm-deep parallel
               beam of E ~ U(1, 18) MeV and a square field of side ~ U(2, 15) cm;
               histories log-uniform on [1e6, 5e7]; problem k draws from seed
               1000 + k and transports with Philox seed 2000 + k
The phantom occupies x, y in [-L/2, L/2] and z in [0, L]; beams start at
z = -1 cm travelling along +z.
"""
import numpy as np

from . import PEGS_FILE, ParallelBeam, XYZGeometry

WATER = "H2O521ICRU"
LUNG = "LUNG521ICRU"
BONE = "ICRPBONE521ICRU"
TISSUE = "ICRUTISSUE521ICRU"


def centred_geometry(n, dx, med=0, rhor=None):
    L = n * dx
    b = -L / 2 + dx * np.arange(n + 1)
    return XYZGeometry(b, b, dx * np.arange(n + 1), med, rhor)


def water30(n=30):
    return dict(name="water30", media=[WATER], ecut=0.7, pcut=0.01, geometry=centred_geometry(n, 30.0 / n),
                source=ParallelBeam(charge=0, energy=2.0, position=(0.0, 0.0, -1.0)), histories=int(1e7),
                batches=10, seed=1)


def bremsstrahlung_spectrum(emin=0.1, emax=6.0, nbins=1000):
    edges = np.linspace(emin, emax, nbins + 1)
    c = 0.5 * (edges[1:] + edges[:-1])
    return edges, (1.0 / c) * (1.0 - c / emax)


def slab64(n=64):
    dx = 16.0 / n
    zc = dx * (np.arange(n) + 0.5)
    medz = np.where(zc < 3, 0, np.where(zc < 9, 1, np.where(zc < 11, 2, 0))).astype(np.int32)
    med = np.broadcast_to(medz[:, None, None], (n, n, n)).ravel()
    return dict(name="slab64", media=[WATER, LUNG, BONE], ecut=0.7, pcut=0.01,
                geometry=centred_geometry(n, dx, med),
                source=ParallelBeam(charge=0, spectrum=bremsstrahlung_spectrum(), position=(0.0, 0.0, -1.0),
                                    rectangle=(-5.0, 5.0, -5.0, 5.0)),
                histories=int(1e8), batches=10, seed=2)


def water128e(n=128):
    dx = 25.6 / n
    return dict(name="water128e", media=[WATER], ecut=0.521, pcut=0.01, geometry=centred_geometry(n, dx),
                source=ParallelBeam(charge=-1, energy=20.0, position=(0.0, 0.0, -1.0),
                                    rectangle=(-5.0, 5.0, -5.0, 5.0)),
                histories=int(2e8), batches=10, seed=3)


def perturbed64(n=64, seed=11):
    dx = 19.2 / n
    rng = np.random.default_rng(seed)
    rhor = 1.0 + 0.1 * rng.uniform(-1.0, 1.0, n ** 3)
    return dict(name="perturbed64", media=[WATER], ecut=0.521, pcut=0.01, geometry=centred_geometry(n, dx, 0, rhor),
                source=ParallelBeam(charge=0, energy=6.0, position=(0.0, 0.0, -1.0),
                                    rectangle=(-2.5, 2.5, -2.5, 2.5)),
                histories=int(2e7), batches=10, seed=13)


def pegs_density(name, path=PEGS_FILE):
    """Mass density (g/cm^3) of a medium as written in its PEGS4 block."""
    key = " MEDIUM=" + name
    with open(path) as f:
        for line in f:
            if line.startswith(key) and line[8:32].strip() == name:
                comp = next(f)
                return float(comp.split("RHO=")[1].split(",")[0])
    raise KeyError(name)


def gaussian_field(n, sigma_vox, rng):
    """Zero-mean white noise on an n^3 grid smoothed by a Gaussian of
    `sigma_vox` voxels (periodic, through the FFT)."""
    k = np.fft.fftfreq(n)
    kz, ky, kx = np.meshgrid(k, k, np.fft.rfftfreq(n), indexing="ij")
    filt = np.exp(-2.0 * (np.pi * sigma_vox) ** 2 * (kx * kx + ky * ky + kz * kz))
    return np.fft.irfftn(np.fft.rfftn(rng.standard_normal((n, n, n))) * filt, s=(n, n, n), axes=(0, 1, 2))


BATCH_MEDIA = [LUNG, WATER, TISSUE, BONE]
BATCH_THRESHOLDS = [0.6, 1.05, 1.4]     # g/cc boundaries between the media above


def batch_problem(k, edge=(32, 160), dx=0.2, hist=(1e6, 5e7), scale=1.0, seed0=1000, philox0=2000):
    """Problem k of the batched workload (see the module docstring)."""
    rng = np.random.default_rng(seed0 + k)
    n = int(rng.integers(edge[0], edge[1] + 1))
    charge = 0 if rng.uniform() < 0.5 else -1
    energy = float(rng.uniform(1.0, 18.0))
    side = float(rng.uniform(2.0, 15.0))
    nh = float(np.exp(rng.uniform(np.log(hist[0]), np.log(hist[1]))))
    f = gaussian_field(n, 1.0 / dx, rng)
    rho = 0.2 + 1.7 * (f - f.min()) / max(f.max() - f.min(), 1e-30)
    med = np.searchsorted(BATCH_THRESHOLDS, rho, side="right").astype(np.int32)
    dens = np.array([pegs_density(m) for m in BATCH_MEDIA])
    rhor = rho / dens[med]
    h = side / 2
    return dict(geometry=centred_geometry(n, dx, med.ravel(), rhor.ravel()),
                source=ParallelBeam(charge=charge, energy=energy, position=(0.0, 0.0, -1.0),
                                    rectangle=(-h, h, -h, h)),
                seed=philox0 + k, histories=max(1, int(round(nh * scale))), edge=n, rho=rho.ravel())


def batched64(nprob=64, scale=1.0, edge=(32, 160)):
    """The batched workload; `scale` multiplies every problem's histories."""
    return dict(name="batched64", media=BATCH_MEDIA, ecut=0.7, pcut=0.01,
                problems=[batch_problem(k, edge=edge, scale=scale) for k in range(nprob)], batches=10)


WORKLOADS = {"water30": water30, "slab64": slab64, "water128e": water128e, "perturbed64": perturbed64}


def sigma_bar(dose, sigma, frac=0.5):
    """Mean relative 1-sigma over voxels with D > frac * Dmax (the DOSXYZnrc
    MAX20-style population) and the corresponding squared mean."""
    m = dose > frac * dose.max()
    r = sigma[m] / dose[m]
    return float(np.sqrt(np.mean(r * r))), int(m.sum())
