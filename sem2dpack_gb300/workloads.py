"""Synthetic workloads: the benchmark configurations as Par.inp-shaped decks.

All inputs are seeded (numpy PCG64, base seed 20261203 + configuration
index); no external data set is involved.

  plain_psv        P-SV elastic, 100 x 100 elements of 100 m, NGLL=5,
                   rho 2700, vp 5000, vs 2887, vertical Ricker force
                   (f0 = 10 Hz) at the centre, absorbing on all sides, CFL 0.5,
                   2000 steps, 16 receivers on a seeded random line.
  sh_rupture       SH dynamic rupture, 400 x 200 elements of 100 m, NGLL=5,
                   rho 2670, vs 3464; split-node fault at mid depth along
                   300 elements (friction 1e4 outside), linear slip weakening
                   mu_s 0.68, mu_d 0.52, Dc 0.4 m, normal stress -120 MPa,
                   shear stress 70 MPa plus Gaussian-correlated noise
                   (correlation 500 m, max 2 MPa), 3 km nucleation patch at
                   81 MPa, absorbing on all sides, 6000 steps.
  psv_rsf          P-SV rate-and-state rupture in a random medium (aging law).
  gradient_shots   P-SV gradient workflow: 512 x 512 elements of 25 m,
                   NGLL=5, homogeneous start model 2700/6000/3464, true
                   model with a seeded Gaussian anomaly (+-10 % on vp, vs,
                   rho), 8 Ricker shots (f0 = 8 Hz) near the surface, 128
                   receivers on the free surface, absorbing elsewhere, 4000
                   steps, L2 waveform misfit.
  batch_shots      independent P-SV shots of uneven size (64^2..512^2
                   elements of 25 m, NGLL=5), each with its own 3-8 layer
                   model (vs 1500-4000 m/s, vp = 1.73 vs, rho = 1700 +
                   0.2 vp), a vertical Ricker force (f0 5-20 Hz) at a
                   random interior point and 32 receivers, 3000 steps.
Each builder takes ``scale`` to shrink the mesh (and steps) for tests.
"""
import numpy as np

from . import abi
from .api import Grid, Problem
from .deck import Fault, Material, ParDeck, Receivers, Sources, Time

BASE_SEED = 20261203


def _rng(config_index):
    return np.random.default_rng(BASE_SEED + config_index)


def plain_psv(scale=1.0, nsteps=2000, precision=abi.PRECISION_FP64, nrec=16):
    """Plain P-SV elastic box (the reference's CPU-runnable case)."""
    n = max(2, int(round(100 * scale)))
    L = 100.0 * n
    rng = _rng(0)
    first = rng.uniform(0.1 * L, 0.9 * L, size=2)
    last = rng.uniform(0.1 * L, 0.9 * L, size=2)
    return ParDeck(
        ngll=5, ndof=2, fmax=25.0, xlim=(0.0, L), zlim=(0.0, L), nelem=(n, n),
        materials=[Material(tag=1, rho=2700.0, cp=5000.0, cs=2887.0)],
        absorbing=[1, 2, 3, 4],
        time=Time(kind="leapfrog", courant=0.5, nsteps=nsteps),
        sources=Sources(coords=[(0.5 * L, 0.5 * L)], f0=10.0, onset=0.12, ampli=1.0, angle=0.0),
        receivers=Receivers(number=nrec, first=tuple(first), last=tuple(last), field="V"),
        precision=precision,
    )


def _correlated_noise(rng, x, corr, amp, dx=25.0):
    """Gaussian-filtered white noise sampled at x, scaled to max |.| = amp."""
    x0, x1 = float(np.min(x)) - 4 * corr, float(np.max(x)) + 4 * corr
    xs = np.arange(x0, x1 + dx, dx)
    white = rng.standard_normal(xs.size)
    k = np.arange(-int(4 * corr / dx), int(4 * corr / dx) + 1) * dx
    kern = np.exp(-0.5 * (k / corr) ** 2)
    smooth = np.convolve(white, kern / kern.sum(), mode="same")
    vals = np.interp(x, xs, smooth)
    return vals * (amp / np.max(np.abs(vals)))


def sh_rupture(scale=1.0, nsteps=6000, precision=abi.PRECISION_MIXED, out_every=10, grid_cls=Grid):
    """SH antiplane rupture on a split-node fault with slip weakening.

    The nucleation patch (81 MPa) must exceed the static strength to start
    the rupture; with mu_s = 0.68 (81.6 MPa under 120 MPa) it would not, so
    mu_s is 0.67 (80.4 MPa) inside the patch.
    """
    nx, nz = max(4, int(round(400 * scale))), max(4, int(round(200 * scale)))
    h = 100.0
    Lx, Lz = nx * h, nz * h
    half = 0.5 * min(300 * h * scale if scale < 1 else 300 * h, 0.9 * Lx)
    patch = 1500.0 * min(1.0, scale * 4) if scale < 1 else 1500.0
    deck = ParDeck(
        ngll=5, ndof=1, fmax=10.0, xlim=(0.0, Lx), zlim=(0.0, Lz), nelem=(nx, nz), ezflt=-1,
        materials=[Material(tag=1, rho=2670.0, cp=6000.0, cs=3464.0)],
        absorbing=[1, 2, 3, 4],
        fault=Fault(tags=(5, 6), friction="SWF", swf_kind=1, normal_kind=1, opening=True),
        time=Time(kind="leapfrog", courant=0.5, nsteps=nsteps),
        receivers=Receivers(number=16, first=(0.1 * Lx, 0.5 * Lz + 2000.0 * min(scale * 4, 1.0)),
                            last=(0.9 * Lx, 0.5 * Lz + 2000.0 * min(scale * 4, 1.0)), field="V"),
        precision=precision,
    )
    grid = grid_cls(deck)
    n1, _ = grid.fault_nodes()
    x = grid.coord()[0, n1 - 1]
    xc = 0.5 * Lx
    rng = _rng(1)
    tt = 70.0e6 + _correlated_noise(rng, x, 500.0, 2.0e6)
    inpatch = np.abs(x - xc) <= patch
    tt[inpatch] = 81.0e6
    mus = np.where(np.abs(x - xc) <= half, 0.68, 1.0e4)
    mus[inpatch] = 0.67
    deck.fault.values = {"Tn": -120.0e6, "Tt": tt, "swf_mus": mus, "swf_mud": 0.52, "swf_dc": 0.4}
    # output every out_every steps, every node
    dt_est = 0.5 * (h * (1.0 - np.sqrt(3.0 / 7.0)) / 2.0) / 3464.0
    deck.fault.otd = out_every * dt_est
    return deck, grid


def von_karman_field(rng, nx, nz, dx, corr, hurst, std):
    """Seeded 2-D von Karman random field on a regular grid (FFT synthesis,
    PSD ~ (1 + k^2 a^2)^-(H+1)), zero mean, given standard deviation."""
    kx = np.fft.fftfreq(nx, d=dx) * 2 * np.pi
    kz = np.fft.fftfreq(nz, d=dx) * 2 * np.pi
    k2 = kz[:, None] ** 2 + kx[None, :] ** 2
    amp = (1.0 + k2 * corr * corr) ** (-(hurst + 1.0) / 2.0)
    spec = np.fft.fft2(rng.standard_normal((nz, nx))) * amp
    f = np.real(np.fft.ifft2(spec))
    f -= f.mean()
    return f * (std / f.std())


def _bilinear(field, x0, z0, dx, x, z):
    """Bilinear interpolation on a regular grid, as DIST_HETE1 samples its
    table (distribution_hete1.f90:100-146)."""
    nz, nx = field.shape
    fx = np.clip((x - x0) / dx, 0, nx - 1 - 1e-9)
    fz = np.clip((z - z0) / dx, 0, nz - 1 - 1e-9)
    i, j = np.floor(fx).astype(int), np.floor(fz).astype(int)
    tx, tz = fx - i, fz - j
    return ((1 - tx) * (1 - tz) * field[j, i] + tx * (1 - tz) * field[j, i + 1]
            + (1 - tx) * tz * field[j + 1, i] + tx * tz * field[j + 1, i + 1])


def psv_rsf(scale=1.0, nsteps=10000, precision=abi.PRECISION_MIXED, rsf_kind=2, out_every=10, grid_cls=Grid):
    """In-plane rupture with rate-and-state friction in a random medium.

    Background vp/vs/rho 6000/3464/2670 perturbed by one von Karman field
    (5 % std, 1 km correlation, Hurst 0.3) given at the GLL points; fault at
    mid depth, aging law a=0.008, b=0.012, Dc=0.02 m, V*=1e-6 m/s, f0=0.6 on
    800 elements (velocity strengthening a=0.02, b=0 outside); initial slip
    rate 1e-12 m/s with the state at steady state, shear stress at steady
    state plus a 25 MPa Gaussian perturbation (radius 1.5 km) for nucleation.
    """
    nx, nz = max(4, int(round(1024 * scale))), max(4, int(round(512 * scale)))
    h = 100.0
    Lx, Lz = nx * h, nz * h
    seg = 0.5 * min(800 * h * max(scale, 0.05), 0.9 * Lx)
    deck = ParDeck(
        ngll=5, ndof=2, fmax=10.0, xlim=(0.0, Lx), zlim=(0.0, Lz), nelem=(nx, nz), ezflt=-1,
        materials=[Material(tag=1, hetero=True)],
        absorbing=[1, 2, 3, 4],
        fault=Fault(tags=(5, 6), friction="RSF", rsf_kind=rsf_kind, normal_kind=1, opening=True),
        time=Time(kind="leapfrog", courant=0.5, nsteps=nsteps),
        receivers=Receivers(number=16, first=(0.1 * Lx, 0.5 * Lz + 1500.0),
                            last=(0.9 * Lx, 0.5 * Lz + 1500.0), field="V"),
        precision=precision,
    )
    grid = grid_cls(deck)
    rng = _rng(2)
    dxg = 25.0
    gx, gz = int(Lx / dxg) + 2, int(Lz / dxg) + 2
    xi = von_karman_field(rng, gx, gz, dxg, 1000.0, 0.3, 0.05)
    coord = grid.coord()
    pert = _bilinear(xi, 0.0, 0.0, dxg, coord[0], coord[1])
    ib = grid.ibool() - 1
    pe = pert[ib]  # (ngll, ngll, nelem)
    deck.hetero = {"rho": 2670.0 * (1 + pe), "cp": 6000.0 * (1 + pe), "cs": 3464.0 * (1 + pe)}
    n1, _ = grid.fault_nodes()
    x = coord[0, n1 - 1]
    xc = 0.5 * Lx
    inside = np.abs(x - xc) <= seg
    a = np.where(inside, 0.008, 0.02)
    b = np.where(inside, 0.012, 0.0)
    dc, vstar, f0, v0, sigma = 0.02, 1.0e-6, 0.6, 1.0e-12, -120.0e6
    theta = np.full(x.shape, dc / v0)
    if rsf_kind == 1:
        theta = np.zeros(x.shape)
    mu0 = a * np.arcsinh(v0 / (2 * vstar) * np.exp((f0 + b * np.log(vstar * theta / dc)) / a)) \
        if rsf_kind != 1 else f0 + a * v0 / (v0 + vstar)
    tau = -sigma * mu0 + 25.0e6 * np.exp(-0.5 * ((x - xc) / 1500.0) ** 2)
    deck.fault.values = {"Tn": sigma, "Tt": tau, "V": v0, "rsf_a": a, "rsf_b": b, "rsf_dc": dc,
                         "rsf_vstar": vstar, "rsf_mus": f0, "rsf_theta": theta}
    dt_est = 0.5 * (h * (1.0 - np.sqrt(3.0 / 7.0)) / 2.0) / (6000.0 * 1.25)
    deck.fault.otd = out_every * dt_est
    return deck, grid


def batch_shots(nsim=256, scale=1.0, nsteps=3000, precision=abi.PRECISION_MIXED, seed_index=3):
    """Decks of the batched-shot configuration.

    Element side 25 m, fmax 40 Hz (the resolution check of CHECK_grid holds
    for vs >= 1500 m/s); layer boundaries on element rows (&MESH_CART_DOMAIN
    tags, velocity increasing with depth); absorbing on all four sides; CFL
    0.5; receivers on a line 5 elements below the top.  ``scale`` shrinks
    the element counts (64..512 -> 64*scale..512*scale, at least 4).
    """
    rng = _rng(seed_index)
    h = 25.0
    lo, hi = max(4, int(round(64 * scale))), max(4, int(round(512 * scale)))
    decks = []
    for _ in range(nsim):
        n = int(rng.integers(lo, hi + 1))
        L = n * h
        nl = int(rng.integers(3, 9))
        cuts = np.sort(rng.choice(np.arange(1, n), size=min(nl - 1, n - 1), replace=False))
        bounds = [0] + [int(c) for c in cuts] + [n]
        vs = np.sort(rng.uniform(1500.0, 4000.0, size=len(bounds) - 1))  # slowest at the top
        domains, mats = [], []
        for k in range(len(bounds) - 1):
            # element rows counted from the bottom (1-based): layer 0 at the top
            ez_top = n - bounds[k]
            ez_bot = n - bounds[k + 1] + 1
            domains.append((k + 1, (1, n), (ez_bot, ez_top)))
            vp = 1.73 * vs[k]
            mats.append(Material(tag=k + 1, rho=1700.0 + 0.2 * vp, cp=vp, cs=float(vs[k])))
        f0 = float(rng.uniform(5.0, 20.0))
        src = (float(rng.uniform(0.1, 0.9) * L), float(rng.uniform(0.1, 0.9) * L))
        depth = L - 5 * h
        decks.append(ParDeck(
            ngll=5, ndof=2, fmax=40.0, xlim=(0.0, L), zlim=(0.0, L), nelem=(n, n),
            domains=domains, materials=mats, absorbing=[1, 2, 3, 4],
            time=Time(kind="leapfrog", courant=0.5, nsteps=nsteps),
            sources=Sources(coords=[src], f0=f0, onset=1.2 / f0, ampli=1.0, angle=0.0),
            receivers=Receivers(number=32, first=(0.05 * L, depth), last=(0.95 * L, depth), field="V"),
            precision=precision,
        ))
    return decks


def gradient_shots(scale=1.0, nsteps=4000, precision=abi.PRECISION_MIXED, nshots=8, seed_index=4):
    """(NodeModel of shot k, start model, true model) for the gradient
    workflow; the node models are (LZ, LX) arrays of rho, vp, vs."""
    from .gradient import NodeModel
    rng = _rng(seed_index)
    n = max(8, int(round(512 * scale)))
    h = 25.0
    L = n * h
    xs = np.linspace(0.1 * L, 0.9 * L, nshots)
    models = []
    for k in range(nshots):
        deck = ParDeck(
            ngll=5, ndof=2, fmax=20.0, xlim=(0.0, L), zlim=(0.0, L), nelem=(n, n),
            materials=[Material(tag=1, rho=2700.0, cp=6000.0, cs=3464.0)], absorbing=[1, 2, 4],
            time=Time(kind="leapfrog", dt=0.3e-3, nsteps=nsteps),
            sources=Sources(coords=[(float(xs[k]), L - 4 * h)], f0=8.0, onset=0.15, ampli=1.0e10, angle=0.0),
            receivers=Receivers(number=128, first=(0.02 * L, L), last=(0.98 * L, L), field="V"),
            precision=precision,
        )
        models.append(NodeModel(deck))
    m0 = models[0]
    X, Z = np.meshgrid(np.linspace(0, L, m0.LX), np.linspace(0, L, m0.LZ))
    xc, zc = rng.uniform(0.35 * L, 0.65 * L), rng.uniform(0.35 * L, 0.6 * L)
    g = np.exp(-((X - xc) ** 2 + (Z - zc) ** 2) / (2 * (0.08 * L) ** 2))
    start = [np.full(X.shape, v) for v in (2700.0, 6000.0, 3464.0)]
    signs = rng.choice([-1.0, 1.0], size=3)
    true = [b * (1.0 + 0.1 * sg * g) for b, sg in zip(start, signs)]
    return models, start, true


def build(deck_or_pair):
    """Problem for a deck (or a (deck, grid) pair from a builder)."""
    if isinstance(deck_or_pair, tuple):
        deck, grid = deck_or_pair
        return Problem(deck, grid)
    return Problem(deck_or_pair)


def tpv3_inplane(scale=1.0, nsteps=None, precision=abi.PRECISION_MIXED, grid_cls=Grid):
    """The reference's SCEC TPV3 in-plane example (EXAMPLES/
    TestFlt2D_SCEC_TPV3_inplane/Par.inp) with its element count multiplied
    by `scale` in each direction (the domain stays 35 x 20 km): NGLL=6,
    Newmark, a Kelvin-Voigt band eta = 0.1 exp(-(z/282.094 m)^2) (x dt)
    along a one-sided slip-weakening fault on the bottom side (shear stress
    81.6 MPa within 1.5 km of x = 0, 70 MPa beyond; static friction 0.677
    within 15 km, 1e4 beyond), v = 'D' on the left side, absorbing right and
    top sides.  16 s of simulated time unless `nsteps` is given."""
    from .distributions import Dist
    nx, nz = max(4, int(round(70 * scale))), max(4, int(round(40 * scale)))
    deck = ParDeck(
        ngll=6, ndof=2, fmax=3.0, xlim=(0.0, 35.0e3), zlim=(0.0, 20.0e3), nelem=(nx, nz),
        materials=[Material(tag=1, rho=2670.0, cp=6000.0, cs=3464.0, kv_eta=0.0)],
        absorbing=[2, 3], dirneu=[(4, "N", "D", False)],
        fault=Fault(tags=(1, 0), friction="SWF", swf_kind=1, normal_kind=1, opening=True),
        time=Time(kind="newmark", courant=0.55, total_time=0.0 if nsteps else 16.0, nsteps=nsteps or 0),
        receivers=Receivers(number=10, first=(0.0, 500.0), last=(15.0e3, 500.0), isamp=20, atnode=False,
                            field="V"),
        precision=precision,
    )
    grid = grid_cls(deck)
    xz = grid.coord()
    n1, _ = grid.fault_nodes()
    x, z = xz[0, n1 - 1], xz[1, n1 - 1]
    tt = Dist("PWCONR", {"num": 2}, [1.5e3, 81.6e6, 70.0e6])
    mus = Dist("PWCONR", {"num": 2}, [15.0e3, 0.677, 1.0e4])
    deck.fault.values = {"Tn": -120.0e6, "Tt": tt(x, z), "swf_mus": mus(x, z), "swf_mud": 0.525, "swf_dc": 0.4}
    deck.fault.oxi = (1, 65, 4)
    ib = grid.ibool() - 1
    px, pz = xz[0][ib], xz[1][ib]
    eta = Dist("GAUSSIAN", {"length": [1.0e6, 282.094], "ampli": 0.1}, [])
    shape = ib.shape
    deck.hetero = {"rho": np.full(shape, 2670.0), "cp": np.full(shape, 6000.0), "cs": np.full(shape, 3464.0),
                   "kveta": eta(px.ravel(), pz.ravel()).reshape(shape)}
    deck.materials[0].hetero = True
    return deck, grid
