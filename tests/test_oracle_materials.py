"""The oracle's dispersive materials against physics, checked on the CPU.

0. Gold, Drude + 2 critical points: the FDTD reflectance and transmittance
   of the 1D line's 50 nm slab match the Airy formulas with the reference's
   analytic permittivity gold_ep (Mm/my_matfunctions_mod.f90:8-31) within
   the discretisation error of 1 nm cells (about 1e-2).

The Lorentz-pole materials:

1. The reference codes one recursion twice: the polarisation-current form of
   the *LorentzJp modules (E-form: E += Ku/eps_inf (curl H - ds sum Jp)) and
   the second-order form of si_mod (D-form: E = D - sum S).  The oracle
   restates each literally; on the same Si fit they must give the same fields
   to rounding, in every layout -- which also checks the oracle's E-form curl
   of each layout against the D-form's updateD.
2. Physics: the FDTD reflectance and transmittance of a 50 nm slab match the
   Airy formulas with the analytic permittivity of the fit within the
   discretisation error of 1 nm cells (a few 1e-3).

The reference's own Graphene (Drude + 4 critical points + Raman):

3. A 50 nm slab of the fit, scaled to 1 nm cells by width/ds, against the
   Airy formulas with the scaled analytic permittivity.  Dropping the
   critical points, flipping the sign of their phases or leaving out the
   width scaling each moves R or T by more than 0.2; the FDTD stays within
   1e-2.
4. The Raman term: its change of the spectra is linear in chi3 for small
   chi3, and the 3D module's exact coefficients and the 2D module's central
   ones agree to O(w_nl dt).

The smaller variants:

5. SiL800, the conductive dielectric: a 50 nm slab against the Airy formulas
   with eps_inf + i sigma/(eps0 omega), at the module's sigma and at one
   large enough that leaving it out would move R/T by more than 0.2.
6. SLG_LJp, four poles with the Kerr term: linear in chi3 like the 3-pole
   sheet.  SLG_ndJp (pole weights zero) without the Kerr term is a
   dielectric of eps_inf for the in-plane field.

The single-cell known-answer test (every dispersive update):

7. A uniformly driven periodic grid runs each cell's D -> E update alone
   (problems.config_cell).  The DFT ratio of the increments of D and E is
   the update's discrete permittivity.  It must equal the z-transform of the
   reference's recursion, derived here independently of the time stepping,
   to the window's truncation (<= 1e-7).  It must also approach the
   material's continuous permittivity within the discretisation error:
   first order in dt for the Drude/critical-point updates, far smaller for
   the Lorentz ones.
"""
import numpy as np
import pytest

from fdtd_gpu import abi, problems


def rel_l2(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / np.linalg.norm(np.asarray(b))


def _te():
    return problems.as_te(problems.config_2d_tmz(precision=abi.F64, n=128, ncyl=3, nfreq=8, npml=16)[0])


def _tm():
    return problems.config_2d_tmz(precision=abi.F64, n=128, ncyl=3, nfreq=8, npml=16)[0]


def _3d():
    return problems.config_3d_sphere(precision=abi.F64, n=48, nfreq=4, npml=6, radius=120.0, half=200)[0]


def _1d():
    spec, _ = problems.config_1d_gold(precision=abi.F64)
    return spec


LAYOUTS = {
    "1d": (_1d, 8000, (abi.EX, abi.HZ)),
    "2d_te": (_te, 1500, (abi.EX, abi.EY, abi.HZ)),
    "2d_tm": (_tm, 1500, (abi.EZ, abi.HX, abi.HY)),
    "3d": (_3d, 400, (abi.EX, abi.EY, abi.EZ, abi.HX, abi.HY, abi.HZ)),
}


@pytest.mark.parametrize("layout", sorted(LAYOUTS))
def test_jp_and_s_codings_are_one_recursion(oracle_lib, layout):
    make, steps, comps = LAYOUTS[layout]
    out = []
    for mat in (problems.SI_S, problems.SI_JP):
        spec = problems.swap_gold(make(), mat)
        assert any(m.kind == "lorentz" for m in spec.materials)
        O = oracle_lib.OracleJob(spec, nthreads=4)
        O.step(1, steps)
        fields = np.concatenate([O.get_field(c).ravel() for c in comps])
        mons = [O.get_monitor(q) for q in range(len(spec.monitors))]
        O.close()
        out.append((fields, mons))
    (fs, ms), (fj, mj) = out
    assert np.linalg.norm(fs) > 0
    assert rel_l2(fj, fs) <= 1e-9
    for (rs, is_), (rj, ij) in zip(ms, mj):
        if np.linalg.norm(rs) > 0:
            assert rel_l2(np.concatenate([rj.ravel(), ij.ravel()]), np.concatenate([rs.ravel(), is_.ravel()])) <= 1e-9


@pytest.mark.parametrize("name", ["SI_S", "GOLD_JP", "FILMGOLD_JP"])
def test_slab_rt_matches_airy_formulas(oracle_lib, name):
    mat = getattr(problems, name)
    spec, meta = problems.config_1d_slab(mat, thickness=50)
    O = oracle_lib.OracleJob(spec)
    O.step(1, meta["Nt"])
    sy = [problems.poynting_1d(*O.get_monitor(q), meta["ds"]) for q in range(3)]
    O.close()
    R, T = -sy[1] / sy[0], sy[2] / sy[0]
    Ra, Ta = problems.slab_rt(problems.lorentz_eps(mat, meta["arg"]), 50e-9, meta["arg"])
    assert np.max(np.abs(R - Ra)) <= 5e-3
    assert np.max(np.abs(T - Ta)) <= 5e-3


def test_dielectric_slab_rt_pins_the_gating(oracle_lib):
    """The incident/reflected gate of the 1D line separates the incident pulse
    from the slab's reflection: a lossless eps=4 slab gives the Airy R and T
    and R + T = 1."""
    from fdtd_gpu.spec import box
    spec, meta = problems.config_1d_gold(precision=abi.F64)
    spec.materials = spec.materials[:1]
    spec.add_dielectric(box((0, 2000, 0), (0, 2049, 0)), 4.0)
    O = oracle_lib.OracleJob(spec)
    O.step(1, meta["Nt"])
    sy = [problems.poynting_1d(*O.get_monitor(q), meta["ds"]) for q in range(3)]
    O.close()
    R, T = -sy[1] / sy[0], sy[2] / sy[0]
    Ra, Ta = problems.slab_rt(np.full(len(meta["arg"]), 4.0 + 0j), 50e-9, meta["arg"])
    assert np.max(np.abs(R - Ra)) <= 1e-4
    assert np.max(np.abs(T - Ta)) <= 1e-4
    assert np.max(np.abs(R + T - 1.0)) <= 1e-4


def test_titanium_fit_has_a_growing_pole():
    """The Ti fit's first pole has negative damping: its recursion factor
    (1 - nu dt)/(1 + nu dt) exceeds 1, so the reference's update grows without
    bound in time whatever the time step.  The library takes the parameters as
    given; this records why no Ti run is part of the tests."""
    nu = problems.TI_JP["gamma"][0]
    dt = problems.config_1d_gold()[1]["dt"]
    assert nu < 0 and (1.0 - nu * dt) / (1.0 + nu * dt) > 1.0


def test_gold_slab_rt_matches_analytic_drude2cp(oracle_lib):
    spec, meta = problems.config_1d_gold(precision=abi.F64)
    O = oracle_lib.OracleJob(spec)
    O.step(1, meta["Nt"])
    sy = [problems.poynting_1d(*O.get_monitor(q), meta["ds"]) for q in range(3)]
    O.close()
    R, T = -sy[1] / sy[0], sy[2] / sy[0]
    eps = problems.drude2cp_eps(problems.GOLD_CONFIG, meta["arg"])
    assert eps.imag.min() > 0  # lossy in the exp(-i omega t) convention
    Ra, Ta = problems.slab_rt(eps, 50e-9, meta["arg"])
    assert np.max(np.abs(R - Ra)) <= 2e-2
    assert np.max(np.abs(T - Ta)) <= 2e-2


def _sheet_spec(chi3, layout=None):
    """The graphene configuration (8 x 8 laterally periodic column) with the
    Lorentz-Jp sheet in place of the Drude sheet; the configuration's fields
    are in V/m, so e_scale = 1."""
    spec, meta = problems.config_3d_graphene(precision=abi.F64, nxy=8, nz=384, nfreq=32)
    mat = dict(problems.GRAPHENE_3LJP, chi3=chi3, e_scale=1.0)
    return problems.swap_graphene(spec, mat), meta


def test_lorentz_sheet_kerr_term_scales_with_chi3(oracle_lib):
    """The Kerr term of the Lorentz-Jp sheet changes the transmitted spectrum
    in proportion to chi3 for small chi3 (doubling chi3 doubles the change),
    and the sheet's normal component stays that of vacuum."""
    res = {}
    for chi3 in (0.0, 1e-12, 2e-12):  # the early pulse edge is ~3e4 V/m at the sheet
        spec, _ = _sheet_spec(chi3)
        O = oracle_lib.OracleJob(spec, nthreads=4)
        O.step(1, 2500)
        re, im = O.get_monitor(0)
        res[chi3] = np.concatenate([re.ravel(), im.ravel()])
        ex, ez = O.get_field(abi.EX), O.get_field(abi.EZ)
        O.close()
    d1 = res[1e-12] - res[0.0]
    d2 = res[2e-12] - res[0.0]
    assert np.linalg.norm(d1) > 1e-9 * np.linalg.norm(res[0.0])  # far above rounding (1e-16)
    assert abs(np.linalg.norm(d2) / np.linalg.norm(d1) - 2.0) < 0.05
    assert np.abs(ez).max() <= 1e-12 * np.abs(ex).max()  # normal incidence: the normal component stays empty


def test_graphene_cp_slab_rt_matches_analytic_permittivity(oracle_lib):
    mat = dict(problems.GRAPHENE_4CP, normal_axis=-1)
    spec, meta = problems.config_1d_slab(mat, thickness=50)
    O = oracle_lib.OracleJob(spec)
    O.step(1, meta["Nt"])
    sy = [problems.poynting_1d(*O.get_monitor(q), meta["ds"]) for q in range(3)]
    O.close()
    R, T = -sy[1] / sy[0], sy[2] / sy[0]
    eps = problems.graphene_cp_eps(mat, meta["ds"], meta["arg"])
    Ra, Ta = problems.slab_rt(eps, 50 * meta["ds"], meta["arg"])
    assert np.max(np.abs(R - Ra)) <= 1e-2
    assert np.max(np.abs(T - Ta)) <= 1e-2
    # the check tells the model's parts apart: without the critical points
    # the analytic R/T move far beyond the tolerance
    R0, T0 = problems.slab_rt(problems.graphene_cp_eps(problems.as_first_initialised_3d(mat), meta["ds"], meta["arg"]),
                              50 * meta["ds"], meta["arg"])
    assert max(np.max(np.abs(R0 - Ra)), np.max(np.abs(T0 - Ta))) > 0.1


def test_graphene_cp_raman_linear_in_chi3_and_forms_agree(oracle_lib):
    """A one-cell Graphene sheet on the 1D line (fields ~1e-4 in the line's
    normalised units): the Raman term changes the spectra by ~1e-8 relative,
    far above rounding, in proportion to chi3; the exact (3D) and central (2D)
    Raman coefficients give the same change to O(w_nl dt) ~ 1e-3."""
    res = {}
    for form in (abi.RAMAN_EXACT, abi.RAMAN_CENTRAL):
        for chi3 in (0.0, 1e-3, 2e-3):
            mat = dict(problems.GRAPHENE_4CP, chi3=chi3, w_nl=2 * np.pi * 47.4e12, gamma_nl=1e12, raman_form=form)
            spec, _ = problems.config_1d_slab(mat, thickness=1, steps=8000)
            O = oracle_lib.OracleJob(spec)
            O.step(1, 8000)
            res[(form, chi3)] = np.concatenate([np.concatenate([a.ravel(), b.ravel()])
                                                for a, b in (O.get_monitor(q) for q in range(3))])
            O.close()
    d = {}
    for form in (abi.RAMAN_EXACT, abi.RAMAN_CENTRAL):
        d1 = res[(form, 1e-3)] - res[(form, 0.0)]
        d2 = res[(form, 2e-3)] - res[(form, 0.0)]
        assert np.linalg.norm(d1) > 1e-10 * np.linalg.norm(res[(form, 0.0)])
        assert abs(np.linalg.norm(d2) / np.linalg.norm(d1) - 2.0) < 1e-3
        d[form] = d1
    assert rel_l2(d[abi.RAMAN_CENTRAL], d[abi.RAMAN_EXACT]) < 1e-2


@pytest.mark.parametrize("sigma", [problems.SI_L800["sigma"], 2e5])
def test_conductive_slab_rt_matches_airy_formulas(oracle_lib, sigma):
    mat = dict(problems.SI_L800, sigma=sigma)
    spec, meta = problems.config_1d_slab(mat, thickness=50)
    O = oracle_lib.OracleJob(spec)
    O.step(1, meta["Nt"])
    sy = [problems.poynting_1d(*O.get_monitor(q), meta["ds"]) for q in range(3)]
    O.close()
    R, T = -sy[1] / sy[0], sy[2] / sy[0]
    eps = problems.conductive_eps(mat, meta["arg"])
    Ra, Ta = problems.slab_rt(eps, 50e-9, meta["arg"])
    assert np.max(np.abs(R - Ra)) <= 2e-3
    assert np.max(np.abs(T - Ta)) <= 2e-3


def test_four_pole_sheet_kerr_term_scales_with_chi3(oracle_lib):
    res = {}
    for chi3 in (0.0, 1e-12, 2e-12):
        spec, meta = problems.config_3d_graphene(precision=abi.F64, nxy=8, nz=384, nfreq=32)
        spec = problems.swap_graphene(spec, dict(problems.GRAPHENE_4LJP, chi3=chi3, e_scale=1.0, ez_uses_x_current=0))
        O = oracle_lib.OracleJob(spec, nthreads=4)
        O.step(1, 2500)
        re, im = O.get_monitor(0)
        res[chi3] = np.concatenate([re.ravel(), im.ravel()])
        O.close()
    d1 = res[1e-12] - res[0.0]
    d2 = res[2e-12] - res[0.0]
    assert np.linalg.norm(d1) > 1e-9 * np.linalg.norm(res[0.0])
    assert abs(np.linalg.norm(d2) / np.linalg.norm(d1) - 2.0) < 0.05


def test_nondispersive_sheet_is_a_dielectric_of_eps_inf(oracle_lib):
    """SLG_ndJp without its Kerr term: zero pole weights leave every Jp at
    zero, so under normal incidence (no normal field) the sheet is a
    dielectric of eps_inf."""
    out = []
    for swap in ("nd", "diel"):
        spec, meta = problems.config_3d_graphene(precision=abi.F64, nxy=8, nz=384, nfreq=32)
        if swap == "nd":
            spec = problems.swap_graphene(spec, dict(problems.GRAPHENE_ND_3LJP, chi3=0.0))
        else:
            from fdtd_gpu.spec import Material
            spec.materials = [Material("dielectric", m.region, eps=problems.GRAPHENE_ND_3LJP["eps_inf"])
                              if m.kind == "graphene" else m for m in spec.materials]
        O = oracle_lib.OracleJob(spec, nthreads=4)
        O.step(1, 2500)
        re, im = O.get_monitor(0)
        out.append(np.concatenate([re.ravel(), im.ravel(), O.get_field(abi.EX).ravel()]))
        O.close()
    assert np.linalg.norm(out[1]) > 0
    assert rel_l2(out[0], out[1]) <= 1e-12


# ---- discrete permittivity of each update, as a z-transform ----------------
# A delay of one step multiplies a transform sum_n x(n) e^{i w t_n} by
# zi = e^{i w dt}.  The critical-point terms are complex recursions driven by
# the real E, and E takes the real part of the quotient, so each of their
# transfers splits into the parts of its coefficients (K + conj-K)/2 and
# (K - conj-K)/2i.

def _eps_drude_cp(eps_inf, wd, gd, amp, phi, om, gam, dt, w):
    """E = Re[(D - I + ha S + sum gb_p g_p)/ga]; I += hb E, S = ha S + hb E,
    g_p = gb_p g_p + gc_p E (M3/gold_mod.f90:61-82, M3/graphene_mod.f90:70-100)."""
    zi = np.exp(1j * np.asarray(w) * dt)
    ha, hb = np.exp(-gd * dt), wd * wd * dt / gd
    ga = eps_inf + 0j
    A = -zi * hb / (1 - zi) + ha * hb * zi / (1 - ha * zi)
    B = 0.0
    for a, ph, o, g in zip(amp, phi, om, gam):
        gb, gc = np.exp((-g + 1j * o) * dt), 1j * dt * 2.0 * a * o * np.exp(-1j * ph)
        ga = ga - gc
        K = gb * gc * zi / (1 - gb * zi)
        Kc = np.conj(gb) * np.conj(gc) * zi / (1 - np.conj(gb) * zi)
        A = A + (K + Kc) / 2
        B = B + (K - Kc) / 2j
    wr, wi = (1 / ga).real, (1 / ga).imag
    return (1 - wr * A + wi * B) / wr


def _eps_lorentz(p, dt, w):
    """JP: E += (1/eps_inf)(dD - c0 dt sum Jp), Jp = g1 Jp + g2 (xi E/c0 - P),
    P += dt Jp (M3/goldLorentzJp_mod.f90:60-86); S: E = (D - sum S)/eps_inf,
    S = a S(n-1) + b S(n-2) + c E (M3/si_mod.f90:55-60)."""
    zi = np.exp(1j * np.asarray(w) * dt)
    e = p["eps_inf"] + 0j
    for xi, o, nu in zip(p["delta_eps"], p["omega"], p["gamma"]):
        if p["form"] == abi.LORENTZ_JP:
            g1, g2 = (1 - nu * dt) / (1 + nu * dt), o * o * dt / (1 + nu * dt)
            den = (1 - g1 * zi) + g2 * dt * zi / (1 - zi)
            e = e + dt * zi * g2 * xi / (den * (1 - zi))
        else:
            a, b = (2 - (dt * o) ** 2) / (1 + dt * nu), (dt * nu - 1) / (1 + dt * nu)
            c = xi * (o * dt) ** 2 / (1 + dt * nu)
            e = e + zi * c / (1 - a * zi - b * zi * zi)
    return e


def _eps_conductive(p, dt, w):
    """E = (D - I)/ga, I += gb E (M3/siL800_mod.f90:39-40, 99-100)."""
    zi = np.exp(1j * np.asarray(w) * dt)
    gb = p["sigma"] * dt / problems.EP0
    return p["eps_inf"] + gb + gb * zi / (1 - zi)


def _damped(p):
    """A Lorentz fit with every pole damped (Si's first pole has none), so its
    response dies out inside the window."""
    return dict(p, gamma=tuple(max(g, 0.02 * problems._W) for g in p["gamma"]))


_GCP = dict(problems.GRAPHENE_4CP, normal_axis=-1)
_G633 = problems.GRAPHENE_633
_G633_LIN = dict(eps_inf=_G633["scale"] * (_G633["n"] ** 2 - _G633["k"] ** 2),
                 sigma=np.sqrt(_G633["scale"]) * 4.0 * np.pi * _G633["n"] * _G633["k"] * problems.C0 * problems.EP0
                 / _G633["wavelength"])
_COND = dict(problems.SI_L800, sigma=2e5)
CELL_CASES = {
    # name: (kind, params, discrete eps(dt, w), continuous eps(w), tolerance against the continuous one)
    "gold": ("gold", problems.GOLD_CONFIG,
             lambda dt, w: _eps_drude_cp(*(problems.GOLD_CONFIG[k] for k in ("eps_inf", "omega_d", "gamma_d", "amp",
                                                                              "phi", "omega", "gamma")), dt, w),
             lambda w: problems.drude2cp_eps(problems.GOLD_CONFIG, w), 3e-2),
    "gold_jp": ("lorentz", problems.GOLD_JP, lambda dt, w: _eps_lorentz(problems.GOLD_JP, dt, w),
                lambda w: problems.lorentz_eps(problems.GOLD_JP, w), 1e-3),
    "si_jp": ("lorentz", _damped(problems.SI_JP), lambda dt, w: _eps_lorentz(_damped(problems.SI_JP), dt, w),
              lambda w: problems.lorentz_eps(_damped(problems.SI_JP), w), 1e-3),
    "si_s": ("lorentz", _damped(problems.SI_S), lambda dt, w: _eps_lorentz(_damped(problems.SI_S), dt, w),
             lambda w: problems.lorentz_eps(_damped(problems.SI_S), w), 1e-3),
    "graphene_cp": ("graphene_cp", _GCP,
                    lambda dt, w: _eps_drude_cp(_GCP["eps_inf"], np.sqrt(_GCP["width"] / 1e-9) * _GCP["drude_omega"],
                                                _GCP["drude_gamma"], [_GCP["width"] / 1e-9 * a for a in _GCP["amp"]],
                                                _GCP["phi"], _GCP["omega"], _GCP["gamma"], dt, w),
                    lambda w: problems.graphene_cp_eps(_GCP, 1e-9, w), 1.5e-2),
    "conductive": ("conductive", _COND, lambda dt, w: _eps_conductive(_COND, dt, w),
                   lambda w: problems.conductive_eps(_COND, w), 2e-3),
    # the conduction term's O(dt) offset: ga carries sigma dt/eps0 of which a
    # centred update would hold half (here ~0.018 in eps ~ 7-12)
    "graphene_633": ("graphene_nk", _G633, lambda dt, w: _eps_conductive(_G633_LIN, dt, w),
                     lambda w: problems.graphene_nk_eps(_G633, w), 3e-3),
}


@pytest.mark.parametrize("name", sorted(CELL_CASES))
def test_cell_permittivity_known_answer(oracle_lib, name):
    kind, params, discrete, continuous, tol = CELL_CASES[name]
    w = problems.dft_omegas(400e-9, 900e-9, 50)
    spec, meta = problems.config_cell(kind, params, steps=256000)
    O = oracle_lib.OracleJob(spec)
    O.step(1, meta["Nt"])
    e = O.get_probe(0)[:, 0]
    O.close()
    eps = problems.cell_eps(e, meta, w)
    exact = discrete(meta["dt"], w)
    assert np.max(np.abs(eps - exact) / np.abs(exact)) <= 1e-7
    cont = continuous(w)
    assert np.max(np.abs(eps - cont) / np.abs(cont)) <= tol


def test_graphene_633_kerr_and_raman_linear_in_chi3(oracle_lib):
    """graphene633's Kerr (alpha) and Raman (1 - alpha) parts on a one-cell
    layer of the 1D line: the change of the spectra is linear in chi3, and
    the instantaneous and delayed parts both act."""
    res = {}
    for alpha in (0.0, 1.0):
        for chi3 in (0.0, 1.0, 2.0):  # changes of ~1e-5 (Raman) and ~5e-4 (Kerr): linear
            mat = dict(problems.GRAPHENE_633, chi3=chi3, alpha=alpha, w_nl=2 * np.pi * 47.4e12, gamma_nl=1e12)
            spec, _ = problems.config_1d_slab(mat, thickness=1, steps=8000)
            O = oracle_lib.OracleJob(spec)
            O.step(1, 8000)
            res[(alpha, chi3)] = np.concatenate([np.concatenate([a.ravel(), b.ravel()])
                                                 for a, b in (O.get_monitor(q) for q in range(3))])
            O.close()
    for alpha in (0.0, 1.0):
        d1 = res[(alpha, 1.0)] - res[(alpha, 0.0)]
        d2 = res[(alpha, 2.0)] - res[(alpha, 0.0)]
        assert np.linalg.norm(d1) > 1e-10 * np.linalg.norm(res[(alpha, 0.0)])
        assert abs(np.linalg.norm(d2) / np.linalg.norm(d1) - 2.0) < 1e-3
    assert rel_l2(res[(1.0, 1.0)] - res[(1.0, 0.0)], res[(0.0, 1.0)] - res[(0.0, 0.0)]) > 0.1
