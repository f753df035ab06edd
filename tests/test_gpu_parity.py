"""GPU force path (through the C ABI) against the CPU oracle and the
reference dumps.  Tolerances: FP64 path 1e-10 relative force RMS (the
oracle itself matches cook's dumps to ~1e-12); mixed path 1e-5 relative
force RMS against FP64, the bound the force path is specified to."""
import numpy as np
import pytest

import macsimus_gb300 as M
from golden_cases import CASES, DIPOLE_CASES, load
from oracle import oracle as O

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-5


def rel_rms(a, b):
    return float(np.sqrt(((a - b) ** 2).sum() / (b ** 2).sum()))


def make(case, precision, **kw):
    g, meta, system, ew = load(case)
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     precision=precision, h=meta["params"]["h"], epsc=meta["params"]["epsc"],
                     omegac=meta["omegac"] or 1.2, **kw)
    return g, meta, system, ew, fp


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_forces_vs_oracle_and_reference(case, precision):
    g, meta, system, ew, fp = make(case, precision)
    assert fp.nkvec == meta["QN"]
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    for d in (0, g["r"].shape[0] - 1):
        f, en = fp.forces(g["r"][d], measure=True)
        fo, eo = orc.forces(g["r"][d], nthreads=4)
        tol = 1e-10 if precision == "fp64" else MIXED_TOL
        assert rel_rms(f, fo) < tol
        assert rel_rms(f, g["f"][d]) < max(tol, 2e-10)
        # energies: relative to the Ewald energy scale |E_self| for the
        # electrostatic parts (el is a near-cancellation of r-space and self
        # terms), relative to itself for LJ; FP32 pair sums give ~1e-7..1e-6
        etol = 1e-10 if precision == "fp64" else 2e-6
        for k in ("el", "er", "ek"):
            assert abs(en[k] - eo[k]) <= etol * abs(eo["eself"]), k
        # LJ: a sum of large repulsive and attractive FP32 terms (~1e-6 floor)
        assert abs(en["lj"] - eo["lj"]) <= (1e-10 if precision == "fp64" else 1e-5) * abs(eo["lj"])
        assert abs(en["vir"] - eo["vir"]) <= etol * abs(eo["vir"]) * 10
        for m in range(6):
            assert abs(en["Pvir"][m] - eo["Pvir"][m]) <= 10 * etol * abs(eo["Pvir"][0]), m
    # total potential energy printed by cook for the last step
    etot_tol = 5e-9 * abs(meta["Epot_last"]) if precision == "fp64" else 2e-6 * abs(eo["eself"])
    assert abs(en["el"] + en["lj"] - meta["Epot_last"]) < etot_tol + 1e-3


@pytest.mark.parametrize("case", DIPOLE_CASES)
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_dipole_term(case, precision):
    """Ewald(2)'s dipole term on the device: epsinf = 1, Yeh-Berkowitz along
    z (el.corr=4) and energy only (el.corr=12): forces against cook's dumps
    and the oracle, the term's energy and virial against the oracle"""
    g, meta, system, ew = load(case)
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"],
                     precision=precision, epsinf=ew["epsinf"], dipole_corr=ew["elcorr"])
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"], epsinf=ew["epsinf"],
                   elcorr=ew["elcorr"])
    tol = 1e-10 if precision == "fp64" else MIXED_TOL
    for d in (0, g["r"].shape[0] - 1):
        f, en = fp.forces(g["r"][d], measure=True)
        fo, eo = orc.forces(g["r"][d], nthreads=4)
        assert rel_rms(f, fo) < tol
        assert rel_rms(f, g["f"][d]) < max(tol, 2e-10)
        assert abs(en["edip"] - eo["edip"]) < 1e-9 * eo["edip"]
        etol = 1e-10 if precision == "fp64" else 2e-6
        assert abs(en["el"] - eo["el"]) <= etol * abs(eo["eself"])
        for m in range(6):
            assert abs(en["Pvir"][m] - eo["Pvir"][m]) <= 10 * etol * abs(eo["Pvir"][0]), m
    # the k-space entry point carries the same term
    fk, e = fp.ewald(g["r"][0])
    _, eo = orc.forces(g["r"][0])
    assert abs(e - (eo["ek"] + eo["eself"] + eo["edip"])) < (1e-9 if precision == "fp64" else 2e-6) * abs(eo["eself"])


@pytest.mark.parametrize("cells", [1, 2, 3])
def test_cell_subdivision_does_not_change_forces(cells):
    g, meta, system, ew, fp = make("spce864", "fp64", cells_per_cutoff=cells)
    f, _ = fp.forces(g["r"][0])
    assert rel_rms(f, g["f"][0]) < 2e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cell_list_is_deterministic(precision):
    """the counting-sort cell list (atomic slots, then every cell's sites
    ranked by site index) gives the same order at every evaluation: forces
    and energies bit-identical over repeated evaluations, also after the
    configuration changed in between"""
    g, meta, system, ew, fp = make("brine532", precision)
    f0, e0 = fp.forces(g["r"][0], measure=True)
    for k in range(12):
        if k % 3 == 2:
            fp.forces(g["r"][1])
        f, e = fp.forces(g["r"][0], measure=True)
        assert np.array_equal(f, f0)
        assert e["el"] == e0["el"] and e["lj"] == e0["lj"]


@pytest.mark.parametrize("case", ["spce864", "brine532"])
@pytest.mark.parametrize("variant", [8, 9, 10])
def test_group_pair_kernel_matches_oracle(case, variant):
    """the group pair kernel (pair_variant 8: warps over groups of 8 home
    sites, neighbours pruned against the group's bounding box) and its
    half-shell forms (every pair once, forces in fixed point; 9 lanes on the
    home sites, 10 lanes on the neighbours) give the oracle's forces and
    energies as the cell kernel does"""
    g, meta, system, ew, fc = make(case, "mixed")
    _, _, _, _, fg = make(case, "mixed", pair_variant=variant)
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    for d in (0, g["r"].shape[0] - 1):
        f, en = fg.forces(g["r"][d], measure=True)
        f0, e0 = fc.forces(g["r"][d], measure=True)
        fo, eo = orc.forces(g["r"][d], nthreads=4)
        assert rel_rms(f, fo) < MIXED_TOL
        assert rel_rms(f, f0) < 2e-6
        for k in ("el", "er", "ek"):
            assert abs(en[k] - eo[k]) <= 2e-6 * abs(eo["eself"]), k
        assert abs(en["lj"] - eo["lj"]) <= 1e-5 * abs(eo["lj"])
        for m in range(6):
            assert abs(en["Pvir"][m] - eo["Pvir"][m]) <= 2e-5 * abs(eo["Pvir"][0]), m
        # bit-reproducible like the cell kernel
        f2, _ = fg.forces(g["r"][d], measure=True)
        assert np.array_equal(f2, f)


@pytest.mark.parametrize("cells", [2, 3])
@pytest.mark.parametrize("polar", [False, True])
@pytest.mark.parametrize("variant", [8, 9, 10])
def test_group_pair_kernel_full_size(cells, polar, variant):
    """32768 waters (SPC/E, or with Drude shells displaced at random): the
    group kernel and its half-shell forms (Drude builds run the lane-per-home
    half-shell kernel for 10) equal the cell kernel within the mixed
    rounding, for cells of a half and of a third of the cutoff"""
    from macsimus_gb300 import configs
    w = configs.workload("drude32768" if polar else "spce32768", seed=3)
    r = w["r"].copy()
    if polar:
        rng = np.random.default_rng(4)
        r[w["system"].ns:] = rng.normal(0, 0.05, (w["system"].ns, 3)) * \
            (w["system"].qpol != 0)[:, None]
    args = (w["system"], [w["L"]] * 3, w["cutoff"], w["alpha"], w["kappa"])
    f0, e0 = M.ForcePath(*args, precision="mixed", cells_per_cutoff=cells).forces(r, measure=True)
    f1, e1 = M.ForcePath(*args, precision="mixed", cells_per_cutoff=cells,
                         pair_variant=variant).forces(r, measure=True)
    assert rel_rms(f1, f0) < 2e-6
    assert abs(e1["er"] - e0["er"]) < 2e-6 * abs(e0["eself"])
    assert abs(e1["lj"] - e0["lj"]) < 1e-5 * abs(e0["lj"])


@pytest.mark.parametrize("cells", [1, 2, 3])
@pytest.mark.parametrize("variant", [9, 10])
def test_half_shell_kernel_every_pair_once(cells, variant):
    """the half-shell group kernel at every cell subdivision (the column
    (0, 0) from the home cell up, pairs inside a cell from the lower sorted
    index): the oracle's forces, LJ energy and virial, so no pair is missing
    or taken twice"""
    g, meta, system, ew, fh = make("spce864", "mixed", pair_variant=variant,
                                   cells_per_cutoff=cells)
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    f, en = fh.forces(g["r"][0], measure=True)
    fo, eo = orc.forces(g["r"][0], nthreads=4)
    assert rel_rms(f, fo) < MIXED_TOL
    assert abs(en["lj"] - eo["lj"]) <= 1e-5 * abs(eo["lj"])
    assert abs(en["er"] - eo["er"]) <= 2e-6 * abs(eo["eself"])
    assert abs(en["vir"] - eo["vir"]) <= 2e-5 * abs(eo["vir"])


@pytest.mark.parametrize("variant", [8, 9, 10])
def test_group_kernel_md_is_reproducible(variant):
    """MD with the group kernel and its half-shell form: the same trajectory
    bit for bit on every run, with and without measurement (the half-shell
    kernel's fixed-point force sums do not depend on the order in which the
    atomics land)"""
    g, meta, system, ew, fq = make("spce864", "mixed", pair_variant=variant)
    # the measuring kernels round the forces as the plain ones do
    fa, _ = fq.forces(g["r"][0], measure=True)
    fb, _ = fq.forces(g["r"][0], measure=False)
    assert np.array_equal(fa, fb)

    def run(measure):
        _, _, _, _, fp = make("spce864", "mixed", pair_variant=variant)
        fp.md_set_state(g["r"][2], g["r"][2] - g["r"][1])
        for _ in range(4):
            fp.md_steps(5, measure=measure)
        return fp.md_get_state()

    a, b, c = run(True), run(True), run(False)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert np.array_equal(a[0], c[0]) and np.array_equal(a[1], c[1])


def test_ewald_kspace_part():
    g, meta, system, ew, fp = make("spce216", "fp64")
    fk, e = fp.ewald(g["r"][0])
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    _, eo = orc.forces(g["r"][0])
    assert abs(e - (eo["ek"] + eo["eself"])) < 1e-9 * abs(eo["eself"])
    # k-space forces sum to zero (conj(S) S is real)
    assert np.abs(fk.sum(axis=0)).max() < 1e-8 * np.abs(fk).max() * len(fk)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", ["spce216", "tip4p216"])
def test_md_step_matches_reference_trajectory(precision, case):
    """one step from cook's dumps; for TIP4P/2005 the M-site forces go to
    O, H, H before SHAKE and M is placed after it"""
    g, meta, system, ew, fp = make(case, precision)
    R = g["r"]
    fp.md_set_state(R[2], R[2] - R[1])
    en = fp.md_steps(1)
    r, r1 = fp.md_get_state()
    tol = 1e-9 if precision == "fp64" else 1e-6
    assert np.abs(r - R[3]).max() < tol
    assert np.isfinite(en["ekin"]) and en["ekin"] > 0


def test_md_many_steps_conserve_energy_like_fp64():
    """200 leap-frog + SHAKE NVE steps of 216 SPC/E from cook's lattice start:
    the mixed path conserves the total energy as well as the FP64 path does
    (the start is violent, so the FP64 drift itself is the yardstick)"""
    drift = {}
    for precision in ("fp64", "mixed"):
        g, meta, system, ew, fp = make("spce216", precision)
        R = g["r"]
        fp.md_set_state(R[2], R[2] - R[1])
        E = []
        for _ in range(10):
            en = fp.md_steps(20)
            E.append(en["el"] + en["lj"] + en["ekin"])
        E = np.array(E)
        assert np.all(np.isfinite(E))
        drift[precision] = np.abs(E - E[0]).max()
    assert drift["mixed"] < 1.5 * drift["fp64"] + 1e-6 * abs(E[0])


def test_shake_failure_is_reported_not_fatal():
    g, meta, system, ew, fp = make("spce216", "fp64", shake_maxit=2)
    fp2 = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"], precision="fp64",
                      epsc=1e-30, shake_maxit=2)
    fp2.md_set_state(g["r"][2], g["r"][2] - g["r"][1])
    with pytest.raises(M.MGError) as e:
        fp2.md_steps(1)
    assert e.value.code == 3
    # the context stays usable
    f, _ = fp2.forces(g["r"][0])
    assert rel_rms(f, g["f"][0]) < 2e-10


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_translation_invariance(precision):
    g, meta, system, ew, fp = make("brine532", precision)
    f0, e0 = fp.forces(g["r"][0], measure=True)
    f1, e1 = fp.forces(g["r"][0] + np.array([3.3, -7.1, 11.9]), measure=True)
    tol = 1e-10 if precision == "fp64" else MIXED_TOL
    assert rel_rms(f1, f0) < tol
    assert abs(e1["el"] - e0["el"]) < 10 * tol * abs(e0["eself"])


def test_full_size_mixed_within_tolerance_of_fp64():
    """32768 SPC/E waters (the benchmark workload): the mixed path stays within
    the 1e-5 relative force RMS bound of the FP64 path; Newton's third law and
    conj(S)S real make the total force vanish; energies agree."""
    from macsimus_gb300 import configs
    w = configs.workload("spce32768", seed=3)
    args = (w["system"], [w["L"]] * 3, w["cutoff"], w["alpha"], w["kappa"])
    fm, em = M.ForcePath(*args, precision="mixed").forces(w["r"], measure=True)
    fd, ed = M.ForcePath(*args, precision="fp64").forces(w["r"], measure=True)
    assert rel_rms(fm, fd) < MIXED_TOL
    scale = np.sqrt((fd ** 2).sum(axis=1).mean())
    assert np.abs(fd.sum(axis=0)).max() < 1e-6 * scale * np.sqrt(len(fd))
    assert np.abs(fm.sum(axis=0)).max() < 1e-3 * scale * np.sqrt(len(fd))
    assert abs(em["lj"] - ed["lj"]) < 1e-6 * abs(ed["lj"])
    assert abs(em["el"] - ed["el"]) < 1e-6 * abs(ed["eself"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_neighbour_lists_match_direct_cells(precision):
    """Verlet lists (cutoff+skin) give the same forces as re-binned cells"""
    g, meta, system, ew = load("spce864")
    args = (system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    fl, el = M.ForcePath(*args, precision=precision, skin=1.5).forces(g["r"][0], measure=True)
    fc, ec = M.ForcePath(*args, precision=precision, skin=-1).forces(g["r"][0], measure=True)
    assert rel_rms(fl, fc) < (1e-12 if precision == "fp64" else 1e-6)
    assert abs(el["lj"] - ec["lj"]) < 1e-6 * abs(ec["lj"])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_md_with_lists_matches_md_with_cells(precision):
    """20 MD steps with lists (rebuilt on displacement) track the cook-style
    re-binning at every step"""
    g, meta, system, ew = load("spce216")
    kw = dict(precision=precision, h=meta["params"]["h"], epsc=meta["params"]["epsc"],
              omegac=meta["omegac"] or 1.2)
    args = (system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    out = []
    for skin in (1.5, -1):
        fp = M.ForcePath(*args, skin=skin, **kw)
        fp.md_set_state(g["r"][2], g["r"][2] - g["r"][1])
        fp.md_steps(20)
        out.append(fp.md_get_state()[0])
    assert np.abs(out[0] - out[1]).max() < (1e-9 if precision == "fp64" else 1e-5)


def test_skin_violation_is_reported():
    """a list kept for too many steps with a tiny skin is detected"""
    g, meta, system, ew = load("spce216")
    fp = M.ForcePath(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"], precision="fp64",
                     skin=1e-4, nl_every=1000, h=meta["params"]["h"])
    fp.md_set_state(g["r"][2], g["r"][2] - g["r"][1])
    with pytest.raises(M.MGError) as e:
        fp.md_steps(5)
    assert e.value.code == 8


@pytest.mark.parametrize("case", ["spce864", "brine532"])
def test_concurrent_kspace_chain_gives_identical_forces(case):
    """the k-space chain on its own stream (default) and serialised give the
    same forces bit for bit (the k-space part is added once either way)"""
    g, meta, system, ew, fp = make(case, "mixed")
    f1, e1 = fp.forces(g["r"][0], measure=True)
    fp.set_overlap(False)
    f2, e2 = fp.forces(g["r"][0], measure=True)
    assert np.array_equal(f1, f2)
    assert e1["el"] == e2["el"] and e1["lj"] == e2["lj"]


@pytest.mark.parametrize("case", ["tip4p216", "t5r216"])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_dependant_md_chain_matches_oracle(precision, case):
    """five steps on the device against the oracle's chain of forces,
    depend_f, SHAKE and depend_r from the same start: TIP4P/2005 (a linear
    dependant) and the T5R model (two Lone and one Rowlinson dependant)"""
    g, meta, system, ew, fp = make(case, precision)
    p = meta["params"]
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    R = g["r"]
    r, r1 = R[2].copy(), R[2] - R[1]
    fp.md_set_state(r, r1)
    fp.md_steps(5)
    rg, _ = fp.md_get_state()
    for _ in range(5):
        f, _ = orc.forces(r, measure=False, nthreads=4)
        r, r1, it, _ = orc.shake_step(r, r1, O.depend_f(system, f, r), p["h"], eps=p["epsc"],
                                      omega=meta["omegac"] / 2)
        r = O.depend_r(system, O.normalize(system, r, ew["L"]))
    assert np.abs(rg - r).max() < (1e-9 if precision == "fp64" else 2e-6)
    if case == "t5r216":
        # and one step from cook's state gives cook's next positions
        g, meta, system, ew, fp = make(case, precision)
        fp.md_set_state(R[2], R[2] - R[1])
        fp.md_steps(1)
        assert np.abs(fp.md_get_state()[0] - R[3]).max() < (1e-9 if precision == "fp64"
                                                             else 2e-6)


@pytest.mark.parametrize("case", ["spce216", "tip4p216"])
def test_step_wraps_molecules_like_normalize(case):
    """cook wraps molecules after every step (normalize(-1)): the
    configuration translated by -1 A in x and y leaves molecules below
    r0 = 0.15, which the step moves by +L, the dependants with them"""
    g, meta, system, ew, fp = make(case, "fp64")
    p = meta["params"]
    orc = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"])
    R = g["r"]
    r = R[2] + np.array([-1.0, -1.0, 0.0])
    r1 = R[2] - R[1]
    fp.md_set_state(r, r1)
    fp.md_steps(1)
    rg, _ = fp.md_get_state()
    f, _ = orc.forces(r, measure=False, nthreads=4)
    ro, _, _, _ = orc.shake_step(r, r1, O.depend_f(system, f), p["h"], eps=p["epsc"],
                                 omega=meta["omegac"] / 2)
    ro = O.depend_r(system, O.normalize(system, ro, ew["L"]))
    moved = np.abs(ro - (r + r1)).max(axis=1) > 1.0
    assert moved.sum() > 100         # molecules did wrap
    assert np.abs(rg - ro).max() < 1e-9
    # without the wrapping the same step leaves them where they are
    g, meta, system, ew, fp = make(case, "fp64", normalize=False)
    fp.md_set_state(r, r1)
    fp.md_steps(1)
    rn, _ = fp.md_get_state()
    ro2, _, _, _ = orc.shake_step(r, r1, O.depend_f(system, f), p["h"], eps=p["epsc"],
                                  omega=meta["omegac"] / 2)
    assert np.abs(rn - O.depend_r(system, ro2)).max() < 1e-9


@pytest.mark.parametrize("case", ["spce864", "brine532", "tip4p216", "widom500"])
def test_tensor_core_kspace_matches_fp32_cores(case):
    """both Ewald passes on the tensor cores (TF32 split into three products)
    against the FP32-core kernels and the FP64 path: k-space forces and
    energy agree to FP32 accuracy"""
    g, meta, system, ew, tc = make(case, "mixed", kspace_engine=3)
    _, _, _, _, fc = make(case, "mixed", kspace_engine=1)
    _, _, _, _, fd = make(case, "fp64")
    r = g["r"][0]
    fk_tc, e_tc = tc.ewald(r)
    fk_fc, e_fc = fc.ewald(r)
    fk_64, e_64 = fd.ewald(r)
    # the k-space part alone: a few 1e-6 from the FP32 structure factor;
    # the tensor-core passes are no less accurate than the FP32-core ones
    err_tc, err_fc = rel_rms(fk_tc, fk_64), rel_rms(fk_fc, fk_64)
    assert err_tc < 1e-5
    assert err_tc < 1.5 * err_fc + 1e-6
    assert rel_rms(fk_tc, fk_fc) < 1e-5
    # energy from the structure factor of pass 1, to the tolerance of the
    # other mixed-path Ewald energies (2e-6 of the self term); the tensor
    # cores' FP32 accumulation rounds toward zero, |S| comes out about 1e-6
    # low, the FP32 cores' sums have no such bias
    _, eo = O.Oracle(system, ew["L"], ew["cutoff"], ew["alpha"], ew["kappa"]).forces(r)
    assert abs(e_tc - e_64) <= 2e-6 * abs(eo["eself"])
    assert abs(e_fc - e_64) <= 2e-6 * abs(eo["eself"])
    f, _ = tc.forces(r)
    f64, _ = fd.forces(r)
    assert rel_rms(f, f64) < MIXED_TOL


def test_full_size_tensor_core_passes_within_tolerance():
    """both k-space passes on the tensor cores at 32768 waters (98304
    charges, 16700 k-vectors): the full mixed step within the force bound"""
    from macsimus_gb300 import configs
    w = configs.workload("spce32768", seed=1)
    s = w["system"]
    fps = {e: M.ForcePath(s, [w["L"]] * 3, w["cutoff"], w["alpha"], w["kappa"], precision=pr,
                          kspace_engine=e) for e, pr in ((3, "mixed"), (0, "fp64"))}
    f3, _ = fps[3].forces(w["r"])
    f0, _ = fps[0].forces(w["r"])
    assert rel_rms(f3, f0) < MIXED_TOL
