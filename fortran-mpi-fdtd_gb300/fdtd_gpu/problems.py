"""Job specs for the reference's three programs and the benchmark workloads.

The reference derives every run parameter from Fortran ``parameter``
expressions; the helpers here evaluate the same expressions in the same
order in IEEE binary64, so the grid, time step, PML conductivity, source
and DFT frequencies are bit-identical to the reference's (the values its
``out.out`` files print are checked by the tests).

Reference programs (paths inside the reference checkout):
  reference_2d(): FDTDsimulations/2D/air-nanoAntennas_Si02-Sisubstrate/program.f90
  reference_3d(): FDTDsimulations/3D/air-AuAntennasSiO2-Si/program.f90
  reference_1d(): FDTDsimulations/1D/TFSF-air_SLG_SiO2_Sidisp/program.f90
Benchmark workloads: config_1d_gold(), config_2d_tmz(), config_3d_sphere(),
config_3d_graphene().
"""
import math

import numpy as np

from . import abi
from .spec import JobSpec, box, spheres

# Mm/constants_mod.f90:3-12
PI = 4.0 * math.atan(1.0)
EP0 = 8.85418781762039e-12
MU0 = PI * 4e-7
C0 = 1.0 / math.sqrt(EP0 * MU0)
Z0 = math.sqrt(MU0 / EP0)
NANO = 1e-9

# Gold, Drude + 2 critical points (M2/gold_mod.f90:25-31, M3/gold_mod.f90:28-34)
GOLD_REFERENCE = dict(eps_inf=1.1431, omega_d=1.3202e16, gamma_d=1.0805e14,
                      amp=(0.26698, 3.0834), phi=(-1.2371, -1.0968),
                      omega=(3.8711e15, 4.1684e15), gamma=(4.4642e14, 2.4555e15))
# The benchmark configs quote the second critical point's damping as 2.3555e15.
GOLD_CONFIG = dict(GOLD_REFERENCE, gamma=(4.4642e14, 2.3555e15))


# Lorentz-pole fits of the reference's material modules; omega and gamma in
# rad/s, from the (2 pi c0/micro) * (...) tables.
_W = 2.0 * PI * C0 / 1e-6


def _lorentz(form, eps_inf, xi, w, nu):
    return dict(form=form, eps_inf=eps_inf, delta_eps=tuple(xi),
                omega=tuple(_W * x for x in w), gamma=tuple(_W * x for x in nu))


# Si, second-order form (M3/si_mod.f90:32-35, M1/si_mod.f90:25-28; no eps_inf term)
SI_S = _lorentz(abi.LORENTZ_S, 1.0, (8.0, 2.85, -0.107), (3.64, 2.76, 1.73), (0.0, 0.063, 2.5))
# Si, polarisation-current form (M3/siLorentzJp_mod.f90:22-26)
SI_JP = _lorentz(abi.LORENTZ_JP, 1.0, (8.0, 2.85, -0.107), (3.64, 2.76, 1.73), (0.0, 0.063, 2.5))
# Gold 500-800 nm (M3/goldLorentzJp_mod.f90:22-26)
GOLD_JP = _lorentz(abi.LORENTZ_JP, 1.053787, (2.862890, -0.0722398, 367.7668),
                   (-2.445679, 1.480982, 0.3371279), (0.2170955, 0.1429645, 0.02285188))
# Gold film (M3/filmGoldLorentzJp_mod.f90:21-25)
FILMGOLD_JP = _lorentz(abi.LORENTZ_JP, 3.497071, (2.301113, 400.0), (-2.393546, 0.3441309),
                       (0.2460773, 0.02533959))
# Titanium 600-1000 nm (M3/titaniumJp_mod.f90:22-26)
TI_JP = _lorentz(abi.LORENTZ_JP, 1.1, (-12.74873, 0.9605442, 67.66233, 55.0525),
                 (4.36014, -1.261863, 0.4063879, -2.176176), (-5.825585, 0.2087635, 1.246245, 8.059584))


# Graphene sheet, 3-Lorentz 1 nm fit (M3/graphene3LorentzJp1nm_mod.f90:27-31).  The
# module's Kerr parameters are public variables a program would set (none
# does); the values here are a test choice: chi3 1e-18 m^2/V^2, a 40 THz
# line of 1 ps damping, fields scaled by z0 as the module does.
GRAPHENE_3LJP = dict(_lorentz(abi.LORENTZ_JP, 1.023242, (4.957366, 4.455092, 1.905429),
                              (0.573075, 1.713164, 4.598546), (0.368926, 2.42099, 1.35581)),
                     sheet=1, chi3=1e-18, w_nl=2.0 * PI * 40e12, gamma_nl=1e12, e_scale=Z0)
# The same sheet with the poles' weights set to zero: SLG_ndJp
# (M3/NodispersiveGraphene.f90:27-32), only eps_inf and the Kerr term act.
GRAPHENE_ND_3LJP = dict(GRAPHENE_3LJP, delta_eps=(0.0, 0.0, 0.0))
# The 4-Lorentz sheet SLG_LJp (M3/grapheneLorentzJp_mod.f90:27-31), with the
# same Kerr choice; its Ez line takes the x current (ez_uses_x_current, 3D).
GRAPHENE_4LJP = dict(_lorentz(abi.LORENTZ_JP, 1.070682, (-0.163673, 0.843432, -0.170024, -0.121134),
                              (1.642784, 0.807691, 0.934364, 0.525964), (2.267351, 1.018179, 0.621508, 0.033048)),
                     sheet=1, chi3=1e-18, w_nl=2.0 * PI * 40e12, gamma_nl=1e12, e_scale=Z0, ez_uses_x_current=1)
# The 1D graphene at 633 nm, graphene633 (M1/graphene633_mod.f90:50): its n, k;
# scaleFactor, xi3, alpha, wNL and dnuNL are set by a program (none does): the
# values here are a test choice (no scaling, linear).
GRAPHENE_633 = dict(n=2.731108, k=1.357, wavelength=633e-9, scale=1.0, chi3=0.0, alpha=0.0, w_nl=0.0, gamma_nl=0.0)


def graphene_nk_eps(p, omega):
    """The permittivity of graphene633's linear update: eps_inf + i sigma/(eps0 w)
    with its sigma and eps_inf from n, k (M1/graphene633_mod.f90:51-52)."""
    sigma = math.sqrt(p["scale"]) * 4.0 * PI * p["n"] * p["k"] * C0 * EP0 / p["wavelength"]
    return conductive_eps(dict(eps_inf=p["scale"] * (p["n"] ** 2 - p["k"] ** 2), sigma=sigma), omega)


# Conductive Si at 800 nm, SiL800 (M3/siL800_mod.f90:16-17): sigma in S/m.
SI_L800 = dict(eps_inf=3.675 ** 2, sigma=112.8134634)


# The reference's Graphene fit (M3/graphene_mod.f90:33-41, the same in M2 and
# M1): Drude plus four critical points of a 0.34 nm layer, scaled to the cell
# by width/ds.  xi3, wNL and dnuNL have no defaults there; the Raman term is
# off here (chi3 = 0) until a caller sets them.
GRAPHENE_4CP = dict(eps_inf=1.0, drude_omega=5.2796e15, drude_gamma=9e15,
                    amp=(13.1068, 1.8417, 0.4191, 0.7737), phi=(-1.8391, 0.3505, 3.0565, -0.1199),
                    omega=(6.1264e14, 6.6843e15, 5.6289e15, 1.118e16),
                    gamma=(1e14, 7.905e14, 6.7526e14, 1.0005e14),
                    width=3.4e-10, chi3=0.0, w_nl=0.0, gamma_nl=0.0,
                    raman_form=abi.RAMAN_EXACT, normal_axis=1)


def graphene_cp_eps(p, ds, omega):
    """Continuous-time permittivity of the Graphene model at cell size ds:
    the Drude + critical-point form of drude2cp_eps with the amplitudes and
    the Drude weight scaled by s = width/ds (M3/graphene_mod.f90:264-269)."""
    s = p["width"] / ds
    q = dict(eps_inf=p["eps_inf"], omega_d=np.sqrt(s) * p["drude_omega"], gamma_d=p["drude_gamma"],
             amp=[s * a for a in p["amp"]], phi=p["phi"], omega=p["omega"], gamma=p["gamma"])
    return drude2cp_eps(q, omega)


def as_first_initialised_3d(p):
    """The 3D module's Graphene as a first initialize_material leaves it:
    initialize_GrapheneVars copies exp1..4 and expi1..4 into locals before
    setexp sets them (M3/graphene_mod.f90:221-231), so gb_p = gc_p = 0 and
    only the Drude and Raman terms act.  Zero amplitudes give the same
    update (g_p stays 0, gax = eps_inf)."""
    return dict(p, amp=(0.0, 0.0, 0.0, 0.0))


def swap_graphene_cp(spec, material):
    """A copy of ``spec`` whose graphene (Drude) sheets are replaced by the
    reference's Graphene ``material`` on the same boxes."""
    import copy
    from .spec import Material
    s = copy.deepcopy(spec)
    s.materials = [Material("graphene_cp", m.region, params=dict(material)) if m.kind == "graphene" else m
                   for m in s.materials]
    return s


def swap_graphene(spec, material):
    """A copy of ``spec`` whose graphene (Drude) sheets are replaced by the
    Lorentz material ``material`` on the same boxes."""
    import copy
    from .spec import Material
    s = copy.deepcopy(spec)
    s.materials = [Material("lorentz", m.region, params=dict(material)) if m.kind == "graphene" else m
                   for m in s.materials]
    return s


def lorentz_eps(p, omega):
    """Continuous-time permittivity of the Lorentz recursion (both codings):
    P'' + 2 nu P' + w^2 P = w^2 deps E, so eps = eps_inf + sum deps w^2 /
    (w^2 - omega^2 - 2i nu omega) in the exp(-i omega t) convention."""
    omega = np.asarray(omega, dtype=np.float64)
    eps = np.full(omega.shape, p["eps_inf"], dtype=np.complex128)
    for de, w, nu in zip(p["delta_eps"], p["omega"], p["gamma"]):
        eps += de * w * w / (w * w - omega * omega - 2j * nu * omega)
    return eps


def drude2cp_eps(p, omega):
    """Analytic Drude + 2 critical points permittivity, gold_ep of
    Mm/my_matfunctions_mod.f90:8-31 (exp(-i omega t) convention):
    eps_inf - wD^2/(w^2 + i gD w) + sum A W (e^{i phi}/(W - w - i G) +
    e^{-i phi}/(W + w + i G))."""
    w = np.asarray(omega, dtype=np.float64)
    eps = p["eps_inf"] - (p["omega_d"] * p["omega_d"]) / (w * w + 1j * p["gamma_d"] * w)
    for a, ph, om, g in zip(p["amp"], p["phi"], p["omega"], p["gamma"]):
        eps = eps + a * om * (np.exp(1j * ph) / (om - w - 1j * g) + np.exp(-1j * ph) / (om + w + 1j * g))
    return eps


def conductive_eps(p, omega):
    """eps_inf + i sigma/(eps0 omega), the permittivity of SiL800's update
    in the exp(-i omega t) convention."""
    w = np.asarray(omega, dtype=np.float64)
    return p["eps_inf"] + 1j * p["sigma"] / (EP0 * w)


def slab_rt(eps, d, omega):
    """|r|^2 and |t|^2 of a slab of permittivity eps and thickness d in
    vacuum at normal incidence (Airy formulas)."""
    k0 = np.asarray(omega) / C0
    n = np.sqrt(np.asarray(eps, dtype=np.complex128))
    n = np.where(n.imag < 0, -n, n)
    r12 = (1.0 - n) / (1.0 + n)
    t12, t21 = 2.0 / (1.0 + n), 2.0 * n / (1.0 + n)
    ph = np.exp(1j * n * k0 * d)
    den = 1.0 - r12 * r12 * ph * ph
    r = r12 * (1.0 - ph * ph) / den
    t = t12 * t21 * ph / den
    return np.abs(r) ** 2, np.abs(t) ** 2


def fint(x):
    """Fortran real -> integer assignment (truncation toward zero)."""
    return int(x)


def dft_omegas(lambda_init, lambda_end, nfreq):
    """arg(m) of P2/program.f90:111-115,294-298: linear in frequency from
    c/lambda_end with df=(fend-finit)/nfreq (the endpoint is excluded)."""
    finit = C0 / lambda_end
    fend = C0 / lambda_init
    df = (fend - finit) / nfreq
    arg = np.empty(nfreq)
    freq = finit
    for m in range(nfreq):
        arg[m] = 2.0 * PI * freq
        freq = freq + df
    return arg


def pml_sigma_max(order, R0, npml, ds):
    """sigmam=(order+1.d0)*c0*log(1.d0/R0)/(2.d0*npml*ds) (P2/program.f90:93)."""
    return (order + 1.0) * C0 * math.log(1.0 / R0) / (2.0 * npml * ds)


def poynting_2d_te(re, im, ds):
    """Sy = -sum_i (ReHz ReEx + ImHz ImEx) ds per frequency (P2/program.f90:477-530).
    re/im: (2, nfreq, ncell) with components (Ex, Hz)."""
    nf, nc = re.shape[1], re.shape[2]
    out = np.zeros(nf)
    for m in range(nf):
        s = 0.0
        for i in range(nc):
            s = s - ((re[1, m, i] * re[0, m, i]) + (im[1, m, i] * im[0, m, i])) * ds
        out[m] = s
    return out


def poynting_3d_y(re, im, ds):
    """Sy = sum (ReHx ReEz + ImHx ImEz - ReHz ReEx - ImHz ImEx) ds (P3/program.f90:613-685).
    re/im: (4, nfreq, ncell) with components (Ex, Ez, Hx, Hz)."""
    ex, ez, hx, hz = 0, 1, 2, 3
    s = ((re[hx] * re[ez]) + (im[hx] * im[ez]) - (re[hz] * re[ex]) - (im[hz] * im[ex])) * ds
    return s.sum(axis=1)


def poynting_1d(re, im, ds):
    """(-(ReHz ReEx) - (ImHz ImEx)) ds z0 (P1/program.f90:312-332); re/im: (2, nfreq, 1)."""
    return (-(re[1, :, 0] * re[0, :, 0]) - (im[1, :, 0] * im[0, :, 0])) * ds * Z0


# ---------------------------------------------------------------------------
# 2D reference program
# ---------------------------------------------------------------------------
def reference_2d(precision=abi.F64):
    """FDTDsimulations/2D/air-nanoAntennas_Si02-Sisubstrate/program.f90 on one
    domain: 125 x 1266 cells, TE (Hz, Ex, Ey), x periodic, y-slab PML."""
    lambda0 = 633.0 * NANO
    f0 = C0 / lambda0
    Ku = 0.5
    ds = 3.999 * NANO
    dt = Ku * ds / C0
    xreal, yreal = 500.0 * NANO, 5064.0 * NANO
    Xmax, Ymax = 1, 3
    nx, ny = math.floor(xreal / ds), math.floor(yreal / ds)
    ic = nx // 2
    n_y = ny // Ymax
    npmlx = npmly = 10
    order = 3.0
    R0 = math.exp(-16.0)
    sigmam = pml_sigma_max(order, R0, npmly, ds)
    periodoin = 1.0 / f0
    w0 = 2.0 * PI * f0
    beta = 1.0
    st = beta * periodoin
    t0 = 4.0 * st
    sposy = npmly + 2
    freqsteps = 200
    arg = dft_omegas(500e-9, 800e-9, freqsteps)
    ptinx, ptiny = ic, sposy + 2
    n_SiO2, n_Si, n_air = 1.46, 3.88, 1.0
    SiO2_ep, Si_ep, air_ep = n_SiO2 ** 2, n_Si ** 2, n_air ** 2
    # materials (program.f90:185-219), global 1-based ranges
    air = dict(x=(1, nx), y=(npmly, fint(0.8 * ny)))
    goldLength, goldThick = 100.0 * NANO, 20.0 * NANO
    au = dict(x=(fint(ic - 0.5 * math.floor(goldLength / ds) + 1), fint(ic + 0.5 * math.floor(goldLength / ds))),
              y=(air["y"][1] - math.floor(goldThick / ds) + 1, air["y"][1]))
    sio2 = dict(x=(1, nx), y=(air["y"][1] + 1, air["y"][1] + 1 + math.floor(284.0 * NANO / ds) - 1))
    si = dict(x=(1, nx), y=(sio2["y"][1] + 1, ny - npmly))
    ptty = fint(0.5 * (si["y"][0] + si["y"][1]))
    distance4incident = ds * float(air["y"][1] - sposy) + beta * 4.5 * lambda0 / n_air
    vel4incident = C0 / n_air
    time4incident = distance4incident / vel4incident
    tfinStop = math.floor(time4incident / dt)
    Nt = 4 * tfinStop
    dn = int(Nt / 20.0)

    spec = JobSpec(layout=abi.LAYOUT_2D_TE, n=(nx, ny, 1), ku=Ku, dt=dt, ds=ds, periodic=(1, 0, 0),
                   main_lo=(0, npmly - 1, 0), main_hi=(nx - 1, ny - npmly - 1, 0),
                   precision=precision, name="reference_2d")

    def b(m):
        return box((m["x"][0] - 1, m["y"][0] - 1, 0), (m["x"][1] - 1, m["y"][1] - 1, 0))
    # update_E call order: air, Au, SiO2, Si (program.f90:345-348)
    spec.add_dielectric(b(air), air_ep)
    spec.add_gold(b(au), GOLD_REFERENCE)
    spec.add_dielectric(b(sio2), SiO2_ep)
    spec.add_dielectric(b(si), Si_ep)
    spec.pml = dict(mode=abi.PML_REFERENCE, npml=((npmlx, npmlx), (npmly, npmly), (0, 0)),
                    eps_lo=air_ep, eps_hi=Si_ep, sigma_max=sigmam, order=order)
    spec.sources.append(dict(component=abi.EX, lo=(0, sposy - 1, 0), hi=(nx - 1, sposy - 1, 0),
                             amp=1.0, t0=t0, st=st, w0=w0))
    line = lambda j: ((0, j - 1, 0), (nx - 1, j - 1, 0))
    spec.add_monitor(*line(ptiny), (abi.EX, abi.HZ), arg, 1, tfinStop - 1)          # in
    spec.add_monitor(*line(ptiny), (abi.EX, abi.HZ), arg, tfinStop + 1, 2 ** 31 - 1)  # r
    spec.add_monitor(*line(ptty), (abi.EX, abi.HZ), arg, 1, 2 ** 31 - 1)           # t
    spec.add_probe((ptinx - 1, ptiny - 1, 0), (abi.EX, abi.HZ), 1, tfinStop - 1)
    spec.add_probe((ptinx - 1, ptiny - 1, 0), (abi.EX, abi.HZ), tfinStop + 1, 2 ** 31 - 1)
    spec.add_probe((ptinx - 1, ptty - 1, 0), (abi.EX, abi.HZ), 1, 2 ** 31 - 1)
    meta = dict(sigmam=sigmam, dt=dt, ds=ds, Nt=Nt, dn=dn, tfinStop=tfinStop, ic=ic, n_y=n_y,
                ptty=ptty, arg=arg, au=au, air=air, sio2=sio2, si=si, nx=nx, ny=ny,
                probe_cells=[(ptinx - 1, ptiny - 1), (ptinx - 1, ptiny - 1), (ptinx - 1, ptty - 1)],
                probe_first=[1, tfinStop + 1, 1])
    return spec, meta


# ---------------------------------------------------------------------------
# 3D reference program
# ---------------------------------------------------------------------------
def reference_3d(precision=abi.F64, nt=None):
    """FDTDsimulations/3D/air-AuAntennasSiO2-Si/program.f90 on one domain:
    125 x 1266 x 25 cells, x and z periodic, y-slab PML with x/z corner
    profiles, gold strip, Ex plane source, DFT planes of Ex, Ez, Hx, Hz."""
    lambda0 = 633.0 * NANO
    f0 = C0 / lambda0
    Ku = 0.5
    ds = 3.999 * NANO
    dt = Ku * ds / C0
    xreal, yreal, zreal = 500.0 * NANO, 5064.0 * NANO, 25.0 * ds
    Ymax = 6
    nx, ny, nz = math.floor(xreal / ds), math.floor(yreal / ds), math.floor(zreal / ds)
    ic, kc = nx // 2, nz // 2
    npmlx = npmly = npmlz = 10
    order = 3.0
    R0 = math.exp(-16.0)
    sigmam = pml_sigma_max(order, R0, npmly, ds)
    periodoin = 1.0 / f0
    w0 = 2.0 * PI * f0
    beta = 1.0
    st = beta * periodoin
    t0 = 4.0 * st
    sposy = npmly + 2
    arg = dft_omegas(500e-9, 800e-9, 100)
    ptiny = sposy + 2
    n_SiO2, n_Si, n_air = 1.46, 3.88, 1.0
    SiO2_ep, Si_ep, air_ep = n_SiO2 ** 2, n_Si ** 2, n_air ** 2
    air = dict(x=(1, nx), y=(npmly + 1, fint(0.8 * ny)), z=(1, nz))
    goldLength, goldThick = 100.0 * NANO, 20.0 * NANO
    au = dict(x=(fint(ic - 0.5 * math.floor(goldLength / ds) + 1), fint(ic + 0.5 * math.floor(goldLength / ds))),
              y=(air["y"][1] - math.floor(goldThick / ds) + 1, air["y"][1]), z=(1, nz))
    sio2 = dict(x=(1, nx), y=(air["y"][1] + 1, air["y"][1] + 1 + math.floor(284.0 * NANO / ds) - 1), z=(1, nz))
    si = dict(x=(1, nx), y=(sio2["y"][1] + 1, ny - npmly), z=(1, nz))
    ptty = fint(0.5 * (si["y"][1] + si["y"][0]))
    distance4incident = ds * float(air["y"][1] - sposy) + beta * 4.5 * lambda0 / n_air
    time4incident = distance4incident / (C0 / n_air)
    tfinStop = math.floor(time4incident / dt)
    Nt = 4 * tfinStop

    spec = JobSpec(layout=abi.LAYOUT_3D, n=(nx, ny, nz), ku=Ku, dt=dt, ds=ds, periodic=(1, 0, 1),
                   main_lo=(0, npmly, 0), main_hi=(nx - 1, ny - npmly - 1, nz - 1),
                   precision=precision, name="reference_3d")

    def b(m):
        return box((m["x"][0] - 1, m["y"][0] - 1, m["z"][0] - 1), (m["x"][1] - 1, m["y"][1] - 1, m["z"][1] - 1))
    spec.add_dielectric(b(air), air_ep)     # update order: air, Au, SiO2, Si (program.f90:411-414)
    spec.add_gold(b(au), GOLD_REFERENCE)
    spec.add_dielectric(b(sio2), SiO2_ep)
    spec.add_dielectric(b(si), Si_ep)
    spec.pml = dict(mode=abi.PML_REFERENCE, npml=((npmlx, npmlx), (npmly, npmly), (npmlz, npmlz)),
                    eps_lo=air_ep, eps_hi=Si_ep, sigma_max=sigmam, order=order)
    spec.sources.append(dict(component=abi.EX, lo=(0, sposy - 1, 0), hi=(nx - 1, sposy - 1, nz - 1),
                             amp=n_air, t0=t0, st=st, w0=w0))
    plane = lambda j: ((0, j - 1, 0), (nx - 1, j - 1, nz - 1))
    comps = (abi.EX, abi.EZ, abi.HX, abi.HZ)
    spec.add_monitor(*plane(ptiny), comps, arg, 1, tfinStop - 1)
    spec.add_monitor(*plane(ptiny), comps, arg, tfinStop + 1, 2 ** 31 - 1)
    spec.add_monitor(*plane(ptty), comps, arg, 1, 2 ** 31 - 1)
    six = (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ)
    # the per-step records of infld, tfld and rfld (program.f90:441-520)
    spec.add_probe((ic - 1, ptiny - 1, kc - 1), six, 1, tfinStop - 1)
    spec.add_probe((ic - 1, ptty - 1, kc - 1), six, 1, 2 ** 31 - 1)
    spec.add_probe((ic - 1, ptiny - 1, kc - 1), six, tfinStop + 1, 2 ** 31 - 1)
    meta = dict(sigmam=sigmam, dt=dt, ds=ds, Nt=Nt if nt is None else nt, tfinStop=tfinStop, ic=ic, kc=kc,
                ptty=ptty, ptiny=ptiny, arg=arg, nx=nx, ny=ny, nz=nz, dn=int(Nt / 20.0), Ymax=Ymax,
                probe_first=(1, 1, tfinStop + 1))
    return spec, meta


# ---------------------------------------------------------------------------
# 1D reference program
# ---------------------------------------------------------------------------
def reference_1d(precision=abi.F64):
    """FDTDsimulations/1D/TFSF-air_SLG_SiO2_Sidisp/program.f90 on one domain:
    13004 cells, TFSF incident line with its own PML, air/SiO2/Si stack."""
    lambda0 = 633.0 * NANO
    f0 = C0 / lambda0
    ds = 1.0 * NANO
    Ku = 0.99
    dt = Ku * ds / C0
    yreal = 20.0 * lambda0 + 344.0 * NANO
    npos = math.floor(yreal / ds)
    jc = fint(0.5 * npos)
    npml = 10
    air_ep, SiO2_ep, Si_ep = 1.0 ** 2, 1.46 ** 2, 3.772 ** 2
    arg = dft_omegas(200e-9, 1000e-9, 100)
    periodoin = 1.0 / f0
    w0 = 2.0 * PI * f0
    beta = 2.0
    st = beta * periodoin
    t0 = 4.0 * st
    spos = npml + math.floor(10.0 * NANO / ds)
    tfsf_bd = spos + math.floor(5.0 * NANO / ds)
    monitor_pti = tfsf_bd - math.floor(5.0 * NANO / ds)
    monitor_ptr = tfsf_bd + math.floor(5.0 * NANO / ds)
    order = 3.0
    R0 = math.exp(-16.0)
    sigmam = (order + 1.0) * C0 * math.log(1.0 / R0) / (2.0 * npml * ds)
    air = (npml + 1, npml + 1 + math.floor(20.0 * lambda0 / ds) - 1)
    sio2 = (air[1] + 1, air[1] + 1 + math.floor(284.0 * NANO / ds) - 1)
    si = (sio2[1] + 1, npos - npml)
    distance4incident = ds * float(jc)
    time4incident = distance4incident / (C0 / 1.0)
    tfinStop = math.floor(time4incident / dt)
    Nt = 6 * tfinStop + 3 * math.floor(t0 / dt)

    spec = JobSpec(layout=abi.LAYOUT_1D, n=(1, npos, 1), ku=Ku, dt=dt, ds=ds,
                   main_lo=(0, npml, 0), main_hi=(0, npos - npml - 1, 0), precision=precision,
                   name="reference_1d")
    for rng, ep in ((air, air_ep), (sio2, SiO2_ep), (si, Si_ep)):
        spec.add_dielectric(box((0, rng[0] - 1, 0), (0, rng[1] - 1, 0)), ep)
    spec.pml = dict(mode=abi.PML_REFERENCE, npml=((0, 0), (npml, npml), (0, 0)),
                    eps_lo=air_ep, eps_hi=Si_ep, sigma_max=sigmam, order=order)
    spec.tfsf = dict(boundary=tfsf_bd - 1, eps_lo=air_ep, eps_hi=air_ep)
    spec.sources.append(dict(component=abi.EX_INC, lo=(0, spos - 1, 0), hi=(0, spos - 1, 0),
                             amp=1.0, t0=t0, st=st, w0=w0))
    spec.add_monitor((0, monitor_pti - 1, 0), (0, monitor_pti - 1, 0), (abi.EX_INC, abi.HZ_INC), arg)
    spec.add_monitor((0, monitor_ptr - 1, 0), (0, monitor_ptr - 1, 0), (abi.EX, abi.HZ), arg)
    spec.add_probe((0, monitor_pti - 1, 0), (abi.EX_INC, abi.HZ_INC))
    spec.add_probe((0, monitor_ptr - 1, 0), (abi.EX, abi.HZ))
    meta = dict(sigmam=sigmam, dt=dt, ds=ds, Nt=Nt, tfinStop=tfinStop, npos=npos, arg=arg,
                tfsf_bd=tfsf_bd, spos=spos, air=air, sio2=sio2, si=si)
    return spec, meta


# ---------------------------------------------------------------------------
# Benchmark workloads (synthetic, seeded)
# ---------------------------------------------------------------------------
def _pulse(lambda0, beta=1.0):
    f0 = C0 / lambda0
    st = beta / f0
    return dict(t0=4.0 * st, st=st, w0=2.0 * PI * f0)


def config_1d_gold(precision=abi.F64, steps=20000):
    """4000 cells, dz=1 nm, Ku=0.99, 20-cell PML each end, 50 nm gold slab at
    cells 2000-2049, soft source at cell 100 (600 nm, 0.5 fs), DFT points at
    cell 300 (incident/reflected, gated) and 3000 (transmitted), 200
    frequencies over 400-900 nm.  The gate at cell 300 falls midway between
    the incident pulse's tail and the slab's reflection, so the two spectra
    separate (a lossless slab gives R + T = 1 to 1e-5)."""
    N, ds, Ku, npml = 4000, 1e-9, 0.99, 20
    dt = Ku * ds / C0
    order, R0 = 3.0, math.exp(-16.0)
    sigmam = pml_sigma_max(order, R0, npml, ds)
    spec = JobSpec(layout=abi.LAYOUT_1D, n=(1, N, 1), ku=Ku, dt=dt, ds=ds,
                   main_lo=(0, npml, 0), main_hi=(0, N - npml - 1, 0), precision=precision,
                   name="config_1d_gold")
    spec.add_dielectric(box((0, npml, 0), (0, N - npml - 1, 0)), 1.0)
    spec.add_gold(box((0, 2000, 0), (0, 2049, 0)), GOLD_CONFIG)
    spec.pml = dict(mode=abi.PML_REFERENCE, npml=((0, 0), (npml, npml), (0, 0)),
                    eps_lo=1.0, eps_hi=1.0, sigma_max=sigmam, order=order)
    p = _pulse(600e-9)
    p["st"] = 0.5e-15
    p["t0"] = 4.0 * p["st"]
    spec.sources.append(dict(component=abi.EX, lo=(0, 100, 0), hi=(0, 100, 0), amp=1.0, **p))
    arg = dft_omegas(400e-9, 900e-9, 200)
    # gate between the incident pulse's tail passing cell 300 (t0 + 4 st after
    # its peak) and the slab's reflection reaching it (3600 cells of travel)
    t_inc_end = ds * float(300 - 100) / C0 + 2.0 * p["t0"]
    t_ref = ds * float(2 * 2000 - 100 - 300) / C0
    tfin = math.floor(0.5 * (t_inc_end + t_ref) / dt)
    spec.add_monitor((0, 300, 0), (0, 300, 0), (abi.EX, abi.HZ), arg, 1, tfin - 1)
    spec.add_monitor((0, 300, 0), (0, 300, 0), (abi.EX, abi.HZ), arg, tfin + 1, 2 ** 31 - 1)
    spec.add_monitor((0, 3000, 0), (0, 3000, 0), (abi.EX, abi.HZ), arg)
    return spec, dict(Nt=steps, tfinStop=tfin, arg=arg, ds=ds, dt=dt)


def config_cell(kind, params, precision=abi.F64, steps=8000, lambda0=600e-9, st=0.5e-15, layout=abi.LAYOUT_2D_TM):
    """A material cell on its own, for its discrete permittivity.  An 8 x 8
    grid, periodic on both axes, filled with the material and driven by the
    same soft source on every cell, stays uniform: curl H is 0, so each cell
    runs only its D -> E update, at the grid's own Ku.  D(n) is the running
    sum of amp g(t_n), and a probe records E(n) every step; the DFT ratio of
    their increments is the update's permittivity (cell_eps)."""
    ds, Ku, n = 1e-9, 0.5, 8
    dt = Ku * ds / C0
    comp = abi.EZ if layout == abi.LAYOUT_2D_TM else abi.EX
    spec = JobSpec(layout=layout, n=(n, n, 1), ku=Ku, dt=dt, ds=ds, periodic=(1, 1, 0),
                   main_lo=(0, 0, 0), main_hi=(n - 1, n - 1, 0), precision=precision, name="config_cell")
    getattr(spec, "add_" + kind)(box((0, 0, 0), (n - 1, n - 1, 0)), params)
    p = _pulse(lambda0)
    p["st"] = st
    p["t0"] = 4.0 * st
    spec.sources.append(dict(component=comp, lo=(0, 0, 0), hi=(n - 1, n - 1, 0), amp=1.0, **p))
    spec.add_probe((3, 4, 0), (comp,), 1, steps)
    return spec, dict(Nt=steps, dt=dt, src=p)


def cell_eps(e, meta, omega):
    """The discrete permittivity D(w)/E(w) of a config_cell run, from the
    probe's E(n) (n = 1..Nt) and the source's increments of D; the
    increments decay, so the finite DFT does not leak a static tail."""
    dt, p = meta["dt"], meta["src"]
    n = np.arange(1, len(e) + 1)
    t = (n - 1) * dt
    dd = np.exp(-0.5 * ((t - p["t0"]) / p["st"]) ** 2) * np.sin(p["w0"] * t)
    de = np.diff(np.concatenate([[0.0], np.asarray(e, dtype=np.float64)]))
    ph = np.exp(1j * np.outer(np.asarray(omega), t))
    return (ph @ dd) / (ph @ de)


def config_1d_slab(material, lo=2000, thickness=50, precision=abi.F64, steps=20000):
    """config_1d_gold's line with the gold slab replaced by ``material``
    (a Lorentz parameter dict, a Graphene one with "drude_omega" or a
    conductive one with "sigma") over
    cells lo .. lo+thickness-1."""
    spec, meta = config_1d_gold(precision=precision, steps=steps)
    spec.materials = spec.materials[:1]
    region = box((0, lo, 0), (0, lo + thickness - 1, 0))
    if "drude_omega" in material:
        spec.add_graphene_cp(region, material)
    elif "wavelength" in material:
        spec.add_graphene_nk(region, material)
    elif "sigma" in material:
        spec.add_conductive(region, material)
    else:
        spec.add_lorentz(region, material)
    spec.name = "config_1d_slab"
    return spec, meta


def swap_gold(spec, material, kind="lorentz"):
    """A copy of ``spec`` whose gold (Drude+2CP) materials are replaced by
    ``material`` (of ``kind``, Lorentz by default) on the same regions."""
    import copy
    from .spec import Material
    s = copy.deepcopy(spec)
    s.materials = [Material(kind, m.region, params=dict(material)) if m.kind == "gold" else m
                   for m in s.materials]
    return s


def as_te(spec):
    """The TE (Hz, Ex, Ey) counterpart of a 2D TMz spec: Ez sources drive Ex
    and the monitors record (Ex, Hz) in place of (Ez, Hx)."""
    import copy
    s = copy.deepcopy(spec)
    s.layout = abi.LAYOUT_2D_TE
    for src in s.sources:
        if src["component"] == abi.EZ:
            src["component"] = abi.EX
    swap = {abi.EZ: abi.EX, abi.HX: abi.HZ}
    for m in s.monitors:
        m.comps = tuple(swap.get(c, c) for c in m.comps)
    for pr in s.probes:
        pr.comps = tuple(swap.get(c, c) for c in pr.comps)
    s.name = spec.name + "_te"
    return s


def config_tfsf(layout=abi.LAYOUT_2D_TM, precision=abi.F64, n=96, npml=10, margin=10, periodic_x=False,
                scatterer=None, radius=8.0, nfreq=8, eps_line=1.0):
    """A plane wave along +y entering a vacuum grid through a total-field /
    scattered-field box: n^2 (2D) or n^3 (3D) cells of 1 nm, Ku = 0.5,
    split-field PML (none along x when ``periodic_x``, where the box spans x
    end to end and has no x faces).  The incident line is driven at a row
    below the box (600 nm carrier, 0.5 fs width).  ``scatterer``: None, a
    material dict for a centred cylinder/sphere of ``radius`` cells, or
    "gold" (Drude+2CP).  Monitors: a row below the box (scattered field), the
    centre row (total) and a row above it (scattered)."""
    ds, Ku = 1e-9, 0.5
    dt = Ku * ds / C0
    dim3 = layout == abi.LAYOUT_3D
    nz = n if dim3 else 1
    order, R0 = 3.0, math.exp(-16.0)
    sigmam = pml_sigma_max(order, R0, npml, ds)
    spec = JobSpec(layout=layout, n=(n, n, nz), ku=Ku, dt=dt, ds=ds, precision=precision,
                   periodic=(1 if periodic_x else 0, 0, 0), name="config_tfsf")
    spec.add_dielectric(box((0, 0, 0), (n - 1, n - 1, nz - 1)), 1.0)
    px = 0 if periodic_x else npml
    spec.pml = dict(mode=abi.PML_SPLIT, npml=((px, px), (npml, npml), (npml, npml) if dim3 else (0, 0)),
                    eps_lo=1.0, sigma_max=sigmam, order=order)
    c = n / 2.0
    if scatterer is not None:
        reg = spheres([(c, c, c if dim3 else 0.0, radius)])
        if scatterer == "gold":
            spec.add_gold(reg, GOLD_CONFIG)
        else:
            spec.add_lorentz(reg, scatterer)
    m = npml + margin
    lo = (0 if periodic_x else m, m, m if dim3 else 0)
    hi = (n - 1 if periodic_x else n - 1 - m, n - 1 - m, n - 1 - m if dim3 else 0)
    spec.tfsf_box = dict(lo=lo, hi=hi, eps_line=eps_line)
    p = _pulse(600e-9)
    p["st"] = 0.5e-15
    p["t0"] = 4.0 * p["st"]
    ys = npml + margin // 2
    spec.sources.append(dict(component=abi.E_INC, lo=(0, ys, 0), hi=(0, ys, 0), amp=1.0, **p))
    arg = dft_omegas(500e-9, 800e-9, nfreq)
    if layout == abi.LAYOUT_2D_TE:
        comps = (abi.EX, abi.HZ)
    elif layout == abi.LAYOUT_2D_TM:
        comps = (abi.EZ, abi.HX)
    else:
        comps = (abi.EX, abi.EZ, abi.HX, abi.HZ)
    k0, k1 = (m, n - 1 - m) if dim3 else (0, 0)
    for y in (lo[1] - 3, int(c), hi[1] + 3):
        spec.add_monitor((lo[0], y, k0), (hi[0], y, k1), comps, arg)
    return spec, dict(arg=arg, ds=ds, dt=dt, box=(lo, hi), ys=ys)


def cylinders_2d(n=2048, count=40, seed=0, rmin=10, rmax=40, ylo=200, yhi=1948, pml=32):
    """40 non-overlapping gold cylinders: radii uniform in {10..40}, centres
    uniform in x in [pml+r+8, n-pml-r-8], y in [ylo+r+8, yhi-r-8], rejected
    when the gap to an accepted cylinder is below 2 cells."""
    rng = np.random.default_rng(seed)
    out = []
    tries = 0
    while len(out) < count:
        tries += 1
        if tries > 100000:
            raise RuntimeError("cylinder placement failed")
        r = int(rng.integers(rmin, rmax + 1))
        cx = float(rng.uniform(pml + r + 8, n - pml - r - 8))
        cy = float(rng.uniform(ylo + r + 8, yhi - r - 8))
        if all(math.hypot(cx - x, cy - y) - r - q >= 2.0 for x, y, q in out):
            out.append((cx, cy, r))
    return [(x, y, 0.0, float(r)) for x, y, r in out]


def config_2d_tmz(precision=abi.F32, n=2048, steps=10000, ncyl=40, nfreq=100, npml=32, seed=0):
    """2D TMz 2048^2, dx=1 nm, Ku=0.5, 32-cell split-field PML on all faces,
    40 seeded gold cylinders, Ez line source at y=100 (600 nm pulse), line DFT
    of Ez and Hx at y=200 (incident/reflected) and y=1948 (transmitted)."""
    ds, Ku = 1e-9, 0.5
    dt = Ku * ds / C0
    order, R0 = 3.0, math.exp(-16.0)
    sigmam = pml_sigma_max(order, R0, npml, ds)
    spec = JobSpec(layout=abi.LAYOUT_2D_TM, n=(n, n, 1), ku=Ku, dt=dt, ds=ds, precision=precision,
                   main_lo=(npml, npml, 0), main_hi=(n - npml - 1, n - npml - 1, 0),
                   name="config_2d_tmz")
    spec.add_dielectric(box((0, 0, 0), (n - 1, n - 1, 0)), 1.0)
    scale = n / 2048.0
    cyl = cylinders_2d(n=n, count=ncyl, seed=seed, ylo=max(int(200 * scale), npml + 12), yhi=min(int(1948 * scale), n - npml - 4), pml=npml,
                       rmin=max(2, int(10 * scale)), rmax=max(3, int(40 * scale))) if ncyl else []
    if cyl:
        spec.add_gold(spheres(cyl), GOLD_CONFIG)
    spec.pml = dict(mode=abi.PML_SPLIT, npml=((npml, npml), (npml, npml), (0, 0)),
                    eps_lo=1.0, sigma_max=sigmam, order=order)
    # positions of the 2048^2 layout, scaled; at reduced sizes kept clear of the PML
    ys = max(int(100 * scale), npml + 4)
    yin = max(int(200 * scale), ys + 8)
    yt = min(int(1948 * scale), n - npml - 4)
    spec.sources.append(dict(component=abi.EZ, lo=(0, ys, 0), hi=(n - 1, ys, 0), amp=1.0, **_pulse(600e-9)))
    arg = dft_omegas(500e-9, 800e-9, nfreq)
    dist = ds * float(yin + 8 - ys) + 4.5 * 600e-9
    tfin = math.floor(dist / C0 / dt)
    spec.add_monitor((0, yin, 0), (n - 1, yin, 0), (abi.EZ, abi.HX), arg, 1, tfin - 1)
    spec.add_monitor((0, yin, 0), (n - 1, yin, 0), (abi.EZ, abi.HX), arg, tfin + 1, 2 ** 31 - 1)
    spec.add_monitor((0, yt, 0), (n - 1, yt, 0), (abi.EZ, abi.HX), arg)
    return spec, dict(Nt=steps, arg=arg, cylinders=cyl, tfinStop=tfin, ds=ds, dt=dt)


def config_3d_sphere(precision=abi.F32, n=512, steps=8000, nfreq=64, npml=16, radius=40.0, half=70):
    """3D 512^3, dx=1 nm, Ku=0.5, 16-cell split-field PML on all faces, gold
    sphere r=40 at the centre, Ex plane source at z=40, DFT of the tangential
    components on the six faces of the box centre +-70, 64 frequencies."""
    ds, Ku = 1e-9, 0.5
    dt = Ku * ds / C0
    order, R0 = 3.0, math.exp(-16.0)
    sigmam = pml_sigma_max(order, R0, npml, ds)
    spec = JobSpec(layout=abi.LAYOUT_3D, n=(n, n, n), ku=Ku, dt=dt, ds=ds, precision=precision,
                   main_lo=(npml,) * 3, main_hi=(n - npml - 1,) * 3, name="config_3d_sphere")
    spec.add_dielectric(box((0, 0, 0), (n - 1, n - 1, n - 1)), 1.0)
    c = n / 2.0
    spec.add_gold(spheres([(c, c, c, radius * n / 512.0)]), GOLD_CONFIG)
    spec.pml = dict(mode=abi.PML_SPLIT, npml=((npml, npml),) * 3, eps_lo=1.0, sigma_max=sigmam, order=order)
    zs = max(int(40 * n / 512), npml + 4)
    spec.sources.append(dict(component=abi.EX, lo=(0, 0, zs), hi=(n - 1, n - 1, zs), amp=1.0, **_pulse(600e-9)))
    arg = dft_omegas(500e-9, 800e-9, nfreq)
    h = int(half * n / 512)
    lo, hi = int(c) - h, int(c) + h
    tang = {0: (abi.EY, abi.EZ, abi.HY, abi.HZ), 1: (abi.EX, abi.EZ, abi.HX, abi.HZ),
            2: (abi.EX, abi.EY, abi.HX, abi.HY)}
    for axis in range(3):
        for pos in (lo, hi):
            a, bb = [lo, lo, lo], [hi, hi, hi]
            a[axis] = bb[axis] = pos
            spec.add_monitor(tuple(a), tuple(bb), tang[axis], arg)
    return spec, dict(Nt=steps, arg=arg, ds=ds, dt=dt)


def config_3d_graphene(precision=abi.F32, nxy=256, nz=384, steps=12000, nfreq=128, npml=10):
    """3D 256x256x384, dx=2 nm, lateral periodic, PML along z, graphene sheet
    at z=192 (E_F=0.4 eV, tau=0.1 ps, T=300 K, chi3=1e-18 m^2/V^2, Raman 0.3 at
    47.4 THz with 1 ps damping), 1550 nm 100 fs pulse of 1e8 V/m from z=20,
    transmitted DFT of the plane-averaged field at z=300 over 1-3 f0 with 128
    frequencies."""
    ds, Ku = 2e-9, 0.5
    dt = Ku * ds / C0
    order, R0 = 3.0, math.exp(-16.0)
    sigmam = pml_sigma_max(order, R0, npml, ds)
    spec = JobSpec(layout=abi.LAYOUT_3D, n=(nxy, nxy, nz), ku=Ku, dt=dt, ds=ds, precision=precision,
                   periodic=(1, 1, 0), main_lo=(0, 0, npml), main_hi=(nxy - 1, nxy - 1, nz - npml - 1),
                   name="config_3d_graphene")
    spec.add_dielectric(box((0, 0, 0), (nxy - 1, nxy - 1, nz - 1)), 1.0)
    zsheet = nz // 2
    spec.add_graphene(box((0, 0, zsheet), (nxy - 1, nxy - 1, zsheet)),
                      dict(fermi_ev=0.4, tau=0.1e-12, temperature=300.0, chi3=1e-18, raman_frac=0.3,
                           raman_freq=47.4e12, raman_tau=1e-12, thickness=ds, e_scale=1.0))
    spec.pml = dict(mode=abi.PML_SPLIT, npml=((0, 0), (0, 0), (npml, npml)), eps_lo=1.0,
                    sigma_max=sigmam, order=order)
    lam = 1550e-9
    f0 = C0 / lam
    st = 100e-15
    spec.sources.append(dict(component=abi.EX, lo=(0, 0, 20), hi=(nxy - 1, nxy - 1, 20), amp=1e8,
                             t0=4.0 * st, st=st, w0=2.0 * PI * f0))
    arg = 2.0 * PI * f0 * np.linspace(1.0, 3.0, nfreq, endpoint=False)
    zt = int(nz * 300 / 384)
    # the transmitted field of a laterally uniform problem: its plane mean
    spec.add_monitor((0, 0, zt), (nxy - 1, nxy - 1, zt), (abi.EX, abi.EY, abi.HX, abi.HY), arg, mean=True)
    return spec, dict(Nt=steps, arg=arg, ds=ds, dt=dt, zsheet=zsheet)
