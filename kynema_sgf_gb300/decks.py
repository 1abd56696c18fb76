"""Input decks (ParmParse text) for the workloads used by tests and bench.

Every deck uses the reference's keys; the ``ks_init.*`` keys select the
synthetic initial fields (seeded noise) that the reference cannot produce.
"""
import math

TWO_PI = 2.0 * math.pi


def tgv(n=64, steps=20, cfl=0.5, rtol=1e-11):
    """Taylor-Green vortex, Re = 1600, triply periodic cube of side 2 pi."""
    return f"""
geometry.prob_lo = 0 0 0
geometry.prob_hi = {TWO_PI!r} {TWO_PI!r} {TWO_PI!r}
geometry.is_periodic = 1 1 1
amr.n_cell = {n} {n} {n}
amr.max_level = 0
incflo.physics = TaylorGreenVortex
incflo.density = 1.0
transport.viscosity = 0.000625
turbulence.model = Laminar
incflo.use_godunov = 1
incflo.godunov_type = ppm
incflo.diffusion_type = 0
nodal_proj.mg_rtol = {rtol}
time.cfl = {cfl}
time.fixed_dt = -1
time.max_step = {steps}
"""


def mol(deck):
    """The same deck advanced with the MOL predictor-corrector
    (``incflo.use_godunov = false``); the deck's ``time.cfl`` must be <= 0.5."""
    out = deck.replace("incflo.use_godunov = 1\nincflo.godunov_type = ppm\n", "incflo.use_godunov = false\n")
    if out == deck:
        raise ValueError("deck does not select the Godunov scheme")
    return out


def abl(nx=256, ny=256, nz=128, steps=100, dx=20.0, cfl=0.9, seed=42, dz=None):
    """Neutral ABL LES: periodic x/y, wall-model bottom, slip top,
    Smagorinsky Cs = 0.135, geostrophic forcing for 8 m/s with Coriolis;
    cells of dx x dx x dz (dz = dx unless given)."""
    dz = dx if dz is None else dz
    return f"""
geometry.prob_lo = 0 0 0
geometry.prob_hi = {nx * dx} {ny * dx} {nz * dz}
geometry.is_periodic = 1 1 0
amr.n_cell = {nx} {ny} {nz}
amr.max_level = 0
zlo.type = wall_model
zhi.type = slip_wall
incflo.physics = ABL
incflo.density = 1.225
transport.viscosity = 1.8e-5
turbulence.model = Smagorinsky
Smagorinsky_coeffs.Cs = 0.135
ICNS.source_terms = GeostrophicForcing CoriolisForcing
CoriolisForcing.latitude = 45.0
GeostrophicForcing.geostrophic_wind = 8 0 0
ABL.kappa = 0.41
ABL.surface_roughness_z0 = 0.1
ABL.wall_shear_stress_type = moeng
incflo.use_godunov = 1
incflo.godunov_type = ppm
incflo.diffusion_type = 0
time.cfl = {cfl}
time.max_step = {steps}
ks_init.loglaw_utop = 8.0
ks_init.noise_amplitude = 0.5
ks_init.noise_zmax = 300
ks_init.noise_seed = {seed}
"""


def disks(nx=128, ny=128, nz=64, steps=40, dcells=16, cts=(0.75, 0.8, 0.7), seed=7, about_center=1, nr=5, nt=20,
          eps_cells=2.0, cfl=0.9):
    """Periodic box with uniform 8 m/s inflow plus noise and uniform-Ct disks
    spaced along x (Gaussian spreading)."""
    dx = 10.0
    D = dcells * dx
    labels = " ".join("T%d" % i for i in range(len(cts)))
    lines = []
    for i, ct in enumerate(cts):
        x = (0.15 + 0.2 * i) * nx * dx
        lines.append(f"Actuator.T{i}.disk_center = {x} {0.5 * ny * dx} {0.5 * nz * dx}")
        lines.append(f"Actuator.T{i}.thrust_coeff = {ct!r}")
    body = "\n".join(lines)
    return f"""
geometry.prob_lo = 0 0 0
geometry.prob_hi = {nx * dx} {ny * dx} {nz * dx}
geometry.is_periodic = 1 1 1
amr.n_cell = {nx} {ny} {nz}
incflo.physics = FreeStream
incflo.velocity = 8.0 0.0 0.0
incflo.density = 1.225
transport.viscosity = 1.8e-5
turbulence.model = Smagorinsky
Smagorinsky_coeffs.Cs = 0.135
ICNS.source_terms = ActuatorForcing
Actuator.labels = {labels}
Actuator.type = UniformCtDisk
Actuator.UniformCtDisk.rotor_diameter = {D}
Actuator.UniformCtDisk.epsilon = {eps_cells * dx}
Actuator.UniformCtDisk.num_points_r = {nr}
Actuator.UniformCtDisk.num_points_t = {nt}
Actuator.UniformCtDisk.spreading_type = UniformGaussian
Actuator.UniformCtDisk.disk_normal = -1.0 0.0 0.0
Actuator.UniformCtDisk.ks_spread_about_center = {about_center}
{body}
incflo.use_godunov = 1
incflo.godunov_type = ppm
incflo.diffusion_type = 0
time.cfl = {cfl}
time.max_step = {steps}
ks_init.noise_amplitude = 0.2
ks_init.noise_seed = {seed}
"""


def adjoint_c3(nx=128, ny=128, nz=64, dcells=16, seed=7, ct_seed=11, n_disks=3, nr=5, nt=20, eps_cells=2.0,
               dt=1.0, viscosity=1.0, about_center=1, cts=None, crossflow=(0.0, 0.0), noise=0.2):
    """Differentiable configuration (adjoint check): triply periodic box of
    8 x 8 x 4 rotor diameters at 10 m cells, uniform 8 m/s inflow plus
    uniform +-0.2 m/s noise, laminar viscosity, fixed dt (CFL about 0.82) and
    ``n_disks`` uniform-Ct disks of ``dcells`` cells in a row along x at
    1, 2, 3 ... diameters facing the flow (normal -x, the force opposes the
    flow), sampling 0.5 D upstream; Ct drawn from U(0.6, 0.9) with numpy's
    default_rng(ct_seed) unless ``cts`` is given.  ``crossflow`` adds a
    uniform (v, w) to the inflow.  Returns
    (deck, box_lo, box_hi, cts), the box being the wake region from the last
    disk to 5 D downstream, one diameter either side of the axis."""
    import numpy as np

    dx = 10.0
    D = dcells * dx
    if cts is None:
        cts = np.random.default_rng(ct_seed).uniform(0.6, 0.9, n_disks)
    cts = [float(c) for c in cts]
    yc, zc = 0.5 * ny * dx, 0.5 * nz * dx
    labels = " ".join("T%d" % i for i in range(len(cts)))
    lines = []
    for i, ct in enumerate(cts):
        lines.append(f"Actuator.T{i}.disk_center = {(1 + i) * D} {yc} {zc}")
        lines.append(f"Actuator.T{i}.thrust_coeff = {ct!r}")
    body = "\n".join(lines)
    deck = f"""
geometry.prob_lo = 0 0 0
geometry.prob_hi = {nx * dx} {ny * dx} {nz * dx}
geometry.is_periodic = 1 1 1
amr.n_cell = {nx} {ny} {nz}
incflo.physics = FreeStream
incflo.velocity = 8.0 {crossflow[0]} {crossflow[1]}
incflo.density = 1.0
transport.viscosity = {viscosity}
turbulence.model = Laminar
ICNS.source_terms = ActuatorForcing
Actuator.labels = {labels}
Actuator.type = UniformCtDisk
Actuator.UniformCtDisk.rotor_diameter = {D}
Actuator.UniformCtDisk.epsilon = {eps_cells * dx}
Actuator.UniformCtDisk.num_points_r = {nr}
Actuator.UniformCtDisk.num_points_t = {nt}
Actuator.UniformCtDisk.spreading_type = UniformGaussian
Actuator.UniformCtDisk.disk_normal = -1.0 0.0 0.0
Actuator.UniformCtDisk.diameters_to_sample = 0.5
Actuator.UniformCtDisk.ks_spread_about_center = {about_center}
{body}
incflo.use_godunov = 1
incflo.godunov_type = ppm
incflo.diffusion_type = 0
time.fixed_dt = {dt}
time.max_step = 1000000
ks_init.noise_amplitude = {noise}
ks_init.noise_seed = {seed}
"""
    xl = len(cts) * D
    lo = (xl, yc - D, zc - D)
    hi = (min(xl + 5 * D, nx * dx), yc + D, zc + D)
    return deck, lo, hi, cts


def abl_disks(nx=512, ny=512, nz=256, dx=10.0, dz=10.0, dcells=20, ngrid=4, spacing=7.0, dt=0.5, seed=42, ct_seed=11, nr=5, nt=20,
              eps_cells=2.0, precision="mixed", cts=None):
    """ABL with a wind farm (production forward + adjoint run): the physics of
    ``abl`` (wall model, slip top, Smagorinsky, geostrophic + Coriolis forcing
    for 8 m/s, log-law + noise initial field) on nx x ny x nz cells of
    dx x dx x dz (default 10 m cubes: 5120 x 5120 x 2560 m), with
    ngrid x ngrid uniform-Ct disks of ``dcells`` cells
    (D = dcells dx) on a square grid spaced ``spacing`` D, hub height D,
    facing -x, Ct drawn from U(0.6, 0.9) with numpy's default_rng(ct_seed)
    unless ``cts`` is given; fixed dt.  Disk k sits in column k // ngrid
    (x) and row k % ngrid (y).  Returns (deck, box_lo, box_hi, cts), the box
    being the rotor-height layer from the first disk column to 5 D
    downstream over the whole width."""
    import numpy as np

    D = dcells * dx
    n = ngrid * ngrid
    if cts is None:
        cts = np.random.default_rng(ct_seed).uniform(0.6, 0.9, n)
    cts = [float(c) for c in cts]
    labels = " ".join("T%d" % i for i in range(n))
    lines = []
    for k, ct in enumerate(cts):
        x = (0.5 + k // ngrid) * spacing * D
        y = (0.5 + k % ngrid) * spacing * D
        lines.append(f"Actuator.T{k}.disk_center = {x} {y} {D}")
        lines.append(f"Actuator.T{k}.thrust_coeff = {ct!r}")
    body = "\n".join(lines)
    deck = f"""
geometry.prob_lo = 0 0 0
geometry.prob_hi = {nx * dx} {ny * dx} {nz * dz}
geometry.is_periodic = 1 1 0
amr.n_cell = {nx} {ny} {nz}
amr.max_level = 0
zlo.type = wall_model
zhi.type = slip_wall
incflo.physics = ABL
incflo.density = 1.225
transport.viscosity = 1.8e-5
turbulence.model = Smagorinsky
Smagorinsky_coeffs.Cs = 0.135
ICNS.source_terms = GeostrophicForcing CoriolisForcing ActuatorForcing
CoriolisForcing.latitude = 45.0
GeostrophicForcing.geostrophic_wind = 8 0 0
ABL.kappa = 0.41
ABL.surface_roughness_z0 = 0.1
ABL.wall_shear_stress_type = moeng
Actuator.labels = {labels}
Actuator.type = UniformCtDisk
Actuator.UniformCtDisk.rotor_diameter = {D}
Actuator.UniformCtDisk.epsilon = {eps_cells * dx}
Actuator.UniformCtDisk.num_points_r = {nr}
Actuator.UniformCtDisk.num_points_t = {nt}
Actuator.UniformCtDisk.spreading_type = UniformGaussian
Actuator.UniformCtDisk.disk_normal = -1.0 0.0 0.0
Actuator.UniformCtDisk.diameters_to_sample = 1.0
Actuator.UniformCtDisk.ks_spread_about_center = 1
{body}
incflo.use_godunov = 1
incflo.godunov_type = ppm
incflo.diffusion_type = 0
time.fixed_dt = {dt}
time.max_step = 1000000
ks_init.loglaw_utop = 8.0
ks_init.noise_amplitude = 0.5
ks_init.noise_zmax = 300
ks_init.noise_seed = {seed}
ks.precision = {precision}
"""
    x0 = 0.5 * spacing * D
    lo = (x0, 0.0, 0.5 * D)
    hi = (min(x0 + 5 * D, nx * dx), ny * dx, 1.5 * D)
    return deck, lo, hi, cts


def abl_temperature(n=(48, 48, 48), steps=10, diffusion_type=0, fixed_dt=-0.5, cfl=0.95, use_force_cfl=0, size=(1000.0, 1000.0, 1000.0),
                    heights=(650.0, 750.0, 1000.0), values=(300.0, 308.0, 308.75)):
    """Stably stratified ABL with temperature transport, the configuration of
    the reference's abl_godunov regression decks (by default the 1000 m cube,
    Boussinesq buoyancy about 300 K, Coriolis at 41.3 deg, ABLForcing at 90 m
    toward (6.128, 5.142) m/s, Moeng wall model, capping inversion 650-750 m
    with a 3 K/km gradient imposed at the top), PPM Godunov."""
    nx, ny, nz = n
    lx, ly, lz = size
    hs = " ".join(repr(float(h)) for h in heights)
    vs = " ".join(repr(float(v)) for v in values)
    return f"""
time.max_step = {steps}
time.fixed_dt = {fixed_dt}
time.cfl = {cfl}
time.use_force_cfl = {use_force_cfl}
incflo.gravity = 0. 0. -9.81
incflo.density = 1.0
incflo.use_godunov = 1
incflo.godunov_type = ppm
incflo.diffusion_type = {diffusion_type}
transport.viscosity = 1.0e-5
transport.laminar_prandtl = 0.7
transport.turbulent_prandtl = 0.3333
transport.reference_temperature = 300.0
turbulence.model = Smagorinsky
Smagorinsky_coeffs.Cs = 0.135
incflo.physics = ABL
ICNS.source_terms = BoussinesqBuoyancy CoriolisForcing ABLForcing
CoriolisForcing.latitude = 41.3
ABLForcing.abl_forcing_height = 90
incflo.velocity = 6.128355544951824 5.142300877492314 0.0
ABL.temperature_heights = {hs}
ABL.temperature_values = {vs}
ABL.kappa = .41
ABL.surface_roughness_z0 = 0.15
amr.n_cell = {nx} {ny} {nz}
amr.max_level = 0
geometry.prob_lo = 0. 0. 0.
geometry.prob_hi = {lx} {ly} {lz}
geometry.is_periodic = 1 1 0
zlo.type = "wall_model"
zhi.type = "slip_wall"
zhi.temperature_type = "fixed_gradient"
zhi.temperature = 0.003
"""
