"""CUDA path vs the FP64 oracle on the same seeded inputs, through the C ABI.

Tolerances: the plain FP64 form must agree to rounding (1e-10 relative L2);
the mixed form (complex FP32 field) within 1e-5 relative L2 after a few
steps, the accuracy budget of a single FP32 z-step chain.  The acceptance
bound for whole runs is 1e-4 relative L2 field error and 1e-3 fluence error.
"""
import numpy as np
import pytest

from gpu_helpers import (many_species_rates, pair, reference_air_components, rel_l2, rt_input, saturating_rate,
                         step_both, two_species_rates)

pytestmark = pytest.mark.gpu

TOL = {"mixed": 1e-5, "fp64": 1e-10}


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_field_upload_is_the_analytic_signal(gpu_lib, precision):
    inp = rt_input(PLASMA=False)
    g, r = pair(inp, precision)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision] / 10


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_linear_step(gpu_lib, precision):
    inp = rt_input(NONLINEARITY=False, PLASMA=False)
    g, r = pair(inp, precision)
    step_both(g, r, 5, 2e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("alg", ["RK2", "RK3", "RK4"])
def test_kerr_step(gpu_lib, precision, alg):
    inp = rt_input(PLASMA=False, ALG=alg, PPcr=30.0)
    g, r = pair(inp, precision)
    step_both(g, r, 3, 2e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("species", [1, 2])
@pytest.mark.parametrize("rmax", [2.0, 5.0])
def test_plasma_density(gpu_lib, precision, species, rmax):
    """rho(t) and Kdrho(t) of the parallel scan vs the sequential RK solve.
    rmax = 5 mm puts the outer rows below the rate cut-off where the row is
    left at rho0 without a scan."""
    kw = dict(PPcr=150.0, rmax=rmax)
    inp = rt_input(**kw)
    if species == 2:
        inp["p_model"][1]["components"] = two_species_rates()
    g, r = pair(inp, precision, store_plasma=True)
    rho_g, rho_r = g.handle.get_plasma(0), r.handle.get_plasma(0)
    kd_g, kd_r = g.handle.get_plasma(1), r.handle.get_plasma(1)
    assert np.max(rho_r) > 1e-6          # ionisation actually happened
    tol = 1e-5 if precision == "mixed" else 1e-10
    assert rel_l2(rho_g, rho_r) < tol
    assert rel_l2(kd_g, kd_r) < tol
    st_g, st_r = g.handle.analyze(), r.handle.analyze()
    assert st_g["rhomax"] == pytest.approx(st_r["rhomax"], rel=tol)


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_full_step_with_plasma(gpu_lib, precision):
    inp = rt_input(PPcr=150.0, ALG="RK4")
    g, r = pair(inp, precision)
    step_both(g, r, 3, 1e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]
    ag, ar = g.handle.analyze(), r.handle.analyze()
    assert rel_l2(ag["fluence"], ar["fluence"]) < TOL[precision]
    assert ag["energy"] == pytest.approx(ar["energy"], rel=TOL[precision])


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_device_loop_matches_oracle_loop(gpu_lib, precision):
    """fil_run: on-device adaptive dz, stop at zmax (Filament.jl:123-172)."""
    import math
    inp = rt_input(PPcr=60.0, ALG="RK4", dzphimax=0.1, dz_initial=1e-2, zmax=0.03)
    g, r = pair(inp, precision)
    code_g, st_g = g.handle.run(0.0, inp["zmax"], 10 ** 6)
    code_r, st_r = r.handle.run(0.0, inp["zmax"], 10 ** 6)
    assert code_g == code_r == 1
    assert st_g["steps"] == st_r["steps"]
    assert st_g["z"] == pytest.approx(st_r["z"], rel=1e-5)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < 10 * TOL[precision]
    assert st_g["energy"] == pytest.approx(r.handle.analyze()["energy"], rel=1e-5)


def test_device_loop_istop(gpu_lib):
    """Imax > Istop ends the loop after the step that exceeded it."""
    inp = rt_input(PLASMA=False, PPcr=30.0, Istop=1.0, dz_initial=2e-3)
    g, r = pair(inp, "mixed")
    code_g, st_g = g.handle.run(0.0, 1.0, 10 ** 6)
    code_r, st_r = r.handle.run(0.0, 1.0, 10 ** 6)
    assert code_g == code_r == 2
    assert st_g["steps"] == st_r["steps"] == 1


def test_run_nmax(gpu_lib):
    inp = rt_input(PLASMA=False)
    g, _ = pair(inp, "mixed")
    code, st = g.handle.run(0.0, 10.0, 5)
    assert code == 3 and st["steps"] == 5


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_upper_half_spectrum_as_the_reference(gpu_lib, precision):
    """The negative frequencies the time guard creates: kept and propagated
    as the reference does (the default, against the literal oracle), or
    dropped on both sides (FIL_OPT_ANALYTIC_PROJECTION).  A narrow time
    guard makes the upper half large enough that dropping it shows."""
    inp = rt_input(PPcr=150.0, ALG="RK4", tguard=60.0)
    out = {}
    for project in (False, True):
        g, r = pair(inp, precision, project=project)
        step_both(g, r, 4, 1e-3)
        Eg, Er = g.handle.get_field(), r.handle.get_field()
        assert rel_l2(Eg, Er) < TOL[precision]
        out[project] = Er
    # the projection is a change of the method far above the FP64 form's
    # agreement with the oracle
    assert rel_l2(out[True], out[False]) > 100 * TOL["fp64"]


@pytest.mark.parametrize("dht", ["tensor", "simt"])
def test_hankel_paths_agree_with_oracle(gpu_lib, dht):
    """Mixed form with the tcgen05 Hankel GEMMs (default) and with the
    CUDA-core GEMMs, full model, RK4."""
    from filament_gb import _abi
    inp = rt_input(PPcr=150.0, ALG="RK4")
    g, r = pair(inp, "mixed")
    if dht == "simt":
        g.handle.set_option(_abi.OPT_DHT_SIMT, 1)
    step_both(g, r, 4, 1e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL["mixed"]


@pytest.mark.parametrize("dht", ["tensor", "simt"])
def test_linear_energy_drift_at_fp32_floor(gpu_lib, dht):
    """Linear propagation over 60 steps against the FP64 oracle.  A tensor
    core summing the whole K range in FP32 (round toward zero) damps every
    transform by ~7e-6, i.e. ~8e-4 in energy here; the exact-slice GEMM must
    stay at the FP32 floor of the FFTs, like the CUDA-core GEMM."""
    from filament_gb import _abi
    inp = rt_input(NONLINEARITY=False, PLASMA=False, rguard=0.0, tguard=0.0, kguard=90.0, wguard=1e30)
    g, r = pair(inp, "mixed")
    if dht == "simt":
        g.handle.set_option(_abi.OPT_DHT_SIMT, 1)
    e0 = r.handle.analyze()["energy"]
    step_both(g, r, 60, 2e-3)
    eg, er = g.handle.analyze()["energy"], r.handle.analyze()["energy"]
    assert abs(eg - er) / e0 < 2.5e-5
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < 3e-5


def _with_raman(inp, thg):
    from filament_gb.responses import init_raman, raman_response_air
    responses, plasma, keys = inp["p_model"]
    raman = {"init": init_raman, "THG": thg, "n2": 0.5e-23, "raman_response": raman_response_air}
    inp = dict(inp)
    inp["p_model"] = (list(responses) + [raman], plasma, keys)
    return inp


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("thg", [True, False])
def test_raman_step(gpu_lib, precision, thg):
    """raman.jl: delayed response F = (H * x) Re(E), x = Re(E)^2 (THG) or
    3/4 |E|^2, packed with the Kerr channel in one FFT."""
    inp = _with_raman(rt_input(ALG="RK4", PPcr=30.0), thg)
    g, r = pair(inp, precision)
    step_both(g, r, 3, 2e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]


def test_linear_only_rows_keep_parity(gpu_lib):
    """A narrow beam (1/e radius 0.25 mm, 8 Pcr) in a 2 mm Hankel window: the outer
    rows' nonlinear step is below 2^-31 of their spectrum, and the FP32 form
    skips their RK stages (the FP64 form and the oracle compute every row).
    The field must still agree with the oracle at the mixed form's one-step
    tolerance, in single steps and in the device loop."""
    import filament_gb as fg
    inp = rt_input(PPcr=8.0, ALG="RK4", beam_a0=0.25e-3)
    E0 = np.abs(fg.Simulation(inp, make_handle=False).field.E0) ** 2
    ratio = E0.max(axis=1) / E0.max()
    assert np.mean(ratio < 1e-12) > 0.2   # a fifth of the rows or more qualify
    g, r = pair(inp, "mixed")
    step_both(g, r, 4, 1e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL["mixed"]
    inp = rt_input(PPcr=8.0, ALG="RK4", beam_a0=0.25e-3, dzphimax=0.1, dz_initial=1e-2, zmax=0.01)
    g, r = pair(inp, "mixed")
    code_g, st_g = g.handle.run(0.0, inp["zmax"], 10 ** 6)
    code_r, st_r = r.handle.run(0.0, inp["zmax"], 10 ** 6)
    assert code_g == code_r == 1 and st_g["steps"] == st_r["steps"]
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < 10 * TOL["mixed"]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_reference_air_rate_tables(gpu_lib, precision):
    """The reference's own air plasma (examples/RT/air.jl:96-121): N2 and O2
    with the rate tables of multiphoton_N2.tf / multiphoton_O2.tf read from
    file, KDEP = true (K from the tables' local order), rho_nt = 2.5e25,
    RK3 plasma integrator.  Density, loss term and a full RK4 step against
    the oracle."""
    inp = rt_input(PPcr=150.0, ALG="RK4")
    pe = inp["p_model"][1]
    pe["components"] = reference_air_components()
    pe["KDEP"] = True
    pe["rho_nt"] = 2.5e25
    g, r = pair(inp, precision, store_plasma=True)
    assert g.problem.pe.rate_n == 10 and len(g.problem.pe.rho_nt) == 2
    rho_g, rho_r = g.handle.get_plasma(0), r.handle.get_plasma(0)
    kd_g, kd_r = g.handle.get_plasma(1), r.handle.get_plasma(1)
    assert np.max(rho_r) > 1e-6
    tol = TOL[precision]
    assert rel_l2(rho_g, rho_r) < tol
    assert rel_l2(kd_g, kd_r) < tol
    step_both(g, r, 3, 1e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < tol


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("kdep", [True, False])
def test_tabulated_rate_general_branch(gpu_lib, precision, kdep):
    """A rate table that is not a power law (local order 8 falling to 3):
    the device interpolates it by segment search, and with KDEP the loss
    term's K is the slope of the segment the intensity falls in."""
    inp = rt_input(PPcr=150.0, ALG="RK4")
    pe = inp["p_model"][1]
    pe["components"] = [{"fraction": 1.0, "ionization_energy": 12.06, "ionization_rate": saturating_rate()}]
    pe["KDEP"] = kdep
    g, r = pair(inp, precision, store_plasma=True)
    slopes = np.diff(g.problem.pe.rate_ly) / np.diff(g.problem.pe.rate_lx)
    assert slopes.max() - slopes.min() > 3.0       # not a power law
    rho_g, rho_r = g.handle.get_plasma(0), r.handle.get_plasma(0)
    kd_g, kd_r = g.handle.get_plasma(1), r.handle.get_plasma(1)
    assert np.max(rho_r) > 1e-6
    tol = TOL[precision]
    assert rel_l2(rho_g, rho_r) < tol
    assert rel_l2(kd_g, kd_r) < tol
    step_both(g, r, 3, 1e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < tol


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_cubic_without_thg(gpu_lib, precision):
    """cubic.jl:41-46 (THG = false): F = 3/4 |E|^2 Re(E), with plasma."""
    inp = rt_input(PPcr=150.0, ALG="RK4")
    inp["p_model"][0][0]["THG"] = False
    g, r = pair(inp, precision)
    assert g.problem.config.cubic_thg == 0
    step_both(g, r, 3, 1e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < TOL[precision]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_ereal_losses_and_plasma(gpu_lib, precision):
    """EREAL = true in current_losses (current_losses.jl:36-44: the loss
    term divides by Re(E)^2) and in the plasma equation
    (photoionization_avalanche.jl:1-17: the rate's argument is Re(E)^2)."""
    inp = rt_input(PPcr=150.0, ALG="RK4")
    responses = inp["p_model"][0]
    for resp in responses:
        if "EREAL" in resp:
            resp["EREAL"] = True
    inp["p_model"][1]["EREAL"] = True
    g, r = pair(inp, precision, store_plasma=True)
    assert g.problem.config.losses_ereal == 1 and g.problem.config.plasma_ereal == 1
    tol = TOL[precision]
    assert rel_l2(g.handle.get_plasma(0), r.handle.get_plasma(0)) < tol
    assert rel_l2(g.handle.get_plasma(1), r.handle.get_plasma(1)) < tol
    step_both(g, r, 3, 1e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < tol


@pytest.mark.parametrize("form", ["mixed", "mixed_simt", "fp64"])
def test_nonparaxial_prefactor(gpu_lib, form):
    """QPARAXIAL = false (nonlinear_propagators.jl:56-63, 232-241): every RK
    stage's right-hand side goes through the Hankel pair with
    QZ(kt, w) = QZ(w) beta / sqrt(beta^2 - kt^2) and the spectral guard in
    between.  Narrow beam (more transverse spectrum) at 60 Pcr with plasma,
    RK4."""
    from filament_gb import _abi
    import filament_gb as fg
    import oracle
    precision = "fp64" if form == "fp64" else "mixed"
    inp = rt_input(PPcr=60.0, ALG="RK4", QPARAXIAL=False, beam_a0=0.5e-3)
    g, r = pair(inp, precision)
    assert g.problem.config.qparaxial == 0
    if form == "mixed_simt":
        g.handle.set_option(_abi.OPT_DHT_SIMT, 1)
    step_both(g, r, 3, 1e-3)
    Eg, Er = g.handle.get_field(), r.handle.get_field()
    assert rel_l2(Eg, Er) < TOL[precision]
    if precision == "fp64":
        # the paraxial prefactor gives a measurably different field
        inp_p = rt_input(PPcr=60.0, ALG="RK4", QPARAXIAL=True, beam_a0=0.5e-3)
        rp = fg.Simulation(inp_p, binding=oracle.binding())
        z = 0.0
        for _ in range(3):
            z += 1e-3
            rp.handle.step(z, 1e-3)
        assert rel_l2(Eg, rp.handle.get_field()) > 100 * TOL["fp64"]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_nonparaxial_device_loop(gpu_lib, precision):
    """The non-paraxial step inside fil_run's captured graphs, adaptive dz."""
    inp = rt_input(PPcr=60.0, ALG="RK3", QPARAXIAL=False, dzphimax=0.1, dz_initial=1e-2, zmax=0.02)
    g, r = pair(inp, precision)
    code_g, st_g = g.handle.run(0.0, inp["zmax"], 10 ** 6)
    code_r, st_r = r.handle.run(0.0, inp["zmax"], 10 ** 6)
    assert code_g == code_r == 1 and st_g["steps"] == st_r["steps"]
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < 10 * TOL[precision]


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
@pytest.mark.parametrize("species", [3, 4])
def test_more_species(gpu_lib, precision, species):
    """Three and four ionising species (photoionization_avalanche.jl:23-27
    loops over any number): density, loss term and full RK4 steps against
    the oracle."""
    inp = rt_input(PPcr=150.0, ALG="RK4")
    inp["p_model"][1]["components"] = many_species_rates(species)
    g, r = pair(inp, precision, store_plasma=True)
    assert g.problem.config.plasma_ncomp == species
    rho_g, rho_r = g.handle.get_plasma(0), r.handle.get_plasma(0)
    assert np.max(rho_r) > 1e-6
    tol = TOL[precision]
    assert rel_l2(rho_g, rho_r) < tol
    assert rel_l2(g.handle.get_plasma(1), r.handle.get_plasma(1)) < tol
    step_both(g, r, 3, 1e-3)
    assert rel_l2(g.handle.get_field(), r.handle.get_field()) < tol
