"""The Green's-function consumers on the GPU (multimode.py, decompositions.py) against the reference
modules' own outputs (tests/golden/multimode_golden.npz, made by tests/golden/make_golden.py), and
their properties on the engine's Green's function of the benchmark medium (N=1024)."""
import os

import numpy as np
import pytest

import cases

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


def _rel(a, b):
    a, b = np.asarray(a), np.asarray(b)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def g():
    return np.load(os.path.join(HERE, "golden", "multimode_golden.npz"))


@pytest.fixture(scope="module")
def mm(nlm):
    from multimodenonlinearoptics_gb300 import multimode
    return multimode


@pytest.fixture(scope="module")
def dc(nlm):
    from multimodenonlinearoptics_gb300 import decompositions
    return decompositions


def test_transfer_and_covariance_matrices(mm, g):
    C, S = g["in_C"], g["in_S"]
    Z = mm.calcQuadratureGreens(C, S)
    assert isinstance(Z, np.ndarray) and np.array_equal(Z, g["Z"])   # element-wise kernel: bit for bit
    cov = mm.calcCovarianceMtx(Z)
    assert _rel(cov, g["cov"]) < 1e-13
    assert _rel(mm.calcCovarianceMtxABasis(C, S), g["cov_a"]) < 1e-13
    assert _rel(mm.normalizedCov(cov), g["normalized_cov"]) < 1e-12
    assert _rel(mm.incoherentPowerGreens(Z), g["incoherent"]) < 1e-15
    assert _rel(mm.photonMean(cov), g["photon_mean"]) < 1e-12
    assert _rel(mm.photonMeanA(g["cov_a"]), g["photon_mean_a"]) < 1e-12
    assert _rel(mm.photonCov(cov), g["photon_cov"]) < 1e-13
    assert _rel(mm.fullEffectiveAdjacencyMatrix(cov), g["full_adjacency"]) < 1e-12
    assert _rel(mm.covLumpLoss(cov, 0.7), g["lump_scalar"]) < 1e-15
    assert _rel(mm.covLumpLoss(g["cov_a"], g["in_transmission"], abasis=True), g["lump_vector_a"]) < 1e-15
    with pytest.raises(AssertionError, match="det"):
        mm.calcCovarianceMtx(1.01 * Z)


def test_squeezing_sampling_and_domains(mm, g):
    C, S, Z, cov = g["in_C"], g["in_S"], g["Z"], g["cov"]
    assert _rel(mm.calcLOSqueezing(cov, g["in_pump"], tol=1.0), g["lo_squeezing"]) < 1e-12
    with pytest.raises(AssertionError, match="C_xx"):
        mm.calcLOSqueezing(cov, g["in_pump"])
    assert _rel(mm.downSampledCov(Z, 12, g["in_omega"], 2.0), g["downsampled_cov"]) < 1e-13
    assert _rel(mm.downSampledCovABasis(C, S, 12, g["in_omega"], 2.0), g["downsampled_cov_a"]) < 1e-13
    for to_time, suffix in ((True, "time"), (False, "freq")):
        c, s = mm.ftGreens(C, S, to_time)
        assert _rel(c, g["ft_c_" + suffix]) < 1e-13 and _rel(s, g["ft_s_" + suffix]) < 1e-13
    to_xp, from_xp = mm.basisTransforms(5)
    assert np.array_equal(to_xp, g["to_xp"]) and np.array_equal(from_xp, g["from_xp"])
    cc, cs = mm.combineGreens(C, S, C.T, S.conj())
    assert _rel(cc, g["combined_c"]) < 1e-13 and _rel(cs, g["combined_s"]) < 1e-13
    assert _rel(mm.parametricFluorescence(g["in_modes"], g["in_diag"]), g["fluorescence"]) < 1e-13
    assert _rel(mm.effectiveAdjacencyMatrix(g["in_modes"], g["in_diag"]), g["adjacency"]) < 1e-13


def test_bloch_messiah_values_and_vectors(mm, g):
    """Values against the reference; vectors (unique up to signs, and up to rotations between the
    near-degenerate values of this case, 2e-10 apart) through orthogonality and reconstruction."""
    Z = g["Z"]
    assert _rel(mm.blochMessiahEigs(Z), g["bm_eigs"]) < 1e-12
    d, left, right = mm.blochMessiahVecs(Z)
    assert _rel(d, g["bm_diag"]) < 1e-12
    n2 = Z.shape[0]
    assert _rel(left.T @ left, np.eye(n2)) < 1e-13 and _rel(right @ right.T, np.eye(n2)) < 1e-13
    assert _rel(left @ np.diag(d) @ right, Z) < 1e-13
    # the reference's eig-based vectors reconstruct Z only to 7e-7 here (its docstring: "does not work
    # well with degeneracies"); the SVD-based ones above are exact to rounding


def test_decompositions(dc, g):
    u, p = dc.leftPolar(g["in_polar_in"])
    assert _rel(u, g["polar_u"]) < 1e-12 and _rel(p, g["polar_p"]) < 1e-12
    for kind in ("c", "r"):
        src = g["in_sym_complex"] if kind == "c" else g["in_sym_real"]
        lam, U = dc.takagi(src)
        assert _rel(lam, g["takagi_%s_l" % kind]) < 1e-12
        assert _rel(U @ np.diag(lam) @ U.T, src) < 1e-12
        assert _rel(U.conj().T @ U, np.eye(src.shape[0])) < 1e-12
    Z = g["Z"]
    n = Z.shape[0] // 2
    ut, st, v = dc.bloch_messiah(Z, tol=1e-6)
    # values that agree to 9 decimals form one degenerate subspace (rounding=9), which the algorithm
    # rotates with an SVD of its block: st then mixes values up to 1e-9 apart, off the diagonal too,
    # and the mix depends on the SVD implementation
    assert np.max(np.abs(np.diag(st) - np.diag(g["bm_st"]))) < 1e-9
    assert np.max(np.abs(st - np.diag(np.diag(st)))) < 1e-9
    assert _rel(ut @ st @ v, Z) < 1e-12
    om = dc.sympmat(n)
    for q in (ut, v):
        assert _rel(q.T @ q, np.eye(2 * n)) < 1e-12
        # Z itself is symplectic to 2.4e-7 (RK4); the reference's own factors are symplectic to 4.3e-5
        assert _rel(q.T @ om @ q, om) < 1e-4
    with pytest.raises(ValueError, match="not symplectic"):
        dc.bloch_messiah(Z)   # RK4 Green's functions are symplectic to 2.4e-7 here, above the default 1e-10


def test_device_tensors_stay_on_device(mm, g):
    torch = pytest.importorskip("torch")
    C = torch.tensor(g["in_C"], device="cuda")
    S = torch.tensor(g["in_S"], device="cuda")
    Z = mm.calcQuadratureGreens(C, S)
    assert Z.is_cuda and Z.dtype == torch.float64
    cov = mm.calcCovarianceMtx(Z)
    assert cov.is_cuda and _rel(cov.cpu().numpy(), g["cov"]) < 1e-13
    e = mm.blochMessiahEigs(Z)
    assert e.is_cuda and _rel(e.cpu().numpy(), g["bm_eigs"]) < 1e-12


def test_non_square_transfer_matrix(mm, oracle_mm):
    """C and S of several output and input modes (rows != columns); an odd column count takes the
    one-column-per-thread kernel."""
    rng = np.random.default_rng(3)
    for rows, cols in ((6, 10), (5, 7)):
        C = cases.noise(rng, rows * cols, 1.0).reshape(rows, cols)
        S = cases.noise(rng, rows * cols, 1.0).reshape(rows, cols)
        assert np.array_equal(mm.calcQuadratureGreens(C, S), oracle_mm.quadrature_greens(C, S))
        assert _rel(mm.calcCovarianceMtxABasis(C, S), oracle_mm.covariance_abasis(C, S)) < 1e-14


@pytest.fixture(scope="module")
def oracle_mm():
    from oracle import multimode_oracle
    return multimode_oracle


def test_benchmark_green_function_properties(nlm, mm):
    """The engine's Green's function of the benchmark medium (N=1024, nZSteps=1000): unit determinant
    of the covariance, and Bloch-Messiah values in reciprocal pairs s_k s_{2N-1-k} = 1 (symplectic)."""
    from multimodenonlinearoptics_gb300.workloads import GREEN_CONFIG, GREEN_DOMAINS
    med = nlm.Chi2PDC(poling=np.ones(GREEN_DOMAINS), **GREEN_CONFIG)
    C, S = med.computeGreensFunction()
    Z = mm.calcQuadratureGreens(C, S)
    mm.calcCovarianceMtx(Z, tol=1e-6)
    e = mm.blochMessiahEigs(Z)
    assert np.max(np.abs(e * e[::-1] - 1)) < 1e-9
    assert e[-1] > 1 + 1e-5   # weak squeezing: the largest value is 1.000124


def test_large_polar_and_vectors(dc, mm, oracle_mm):
    """Square matrices of 512+ rows take the eigensolver route for the polar factor; both routes
    against the oracle (scipy SVD)."""
    rng = np.random.default_rng(9)
    for n in (40, 600):
        a = np.eye(n) + 0.2 * rng.standard_normal((n, n)) / np.sqrt(n)
        u, p = dc.leftPolar(a)
        ur, pr = oracle_mm.left_polar(a)
        assert _rel(u, ur) < 1e-12 and _rel(p, pr) < 1e-12
        assert _rel(p @ u, a) < 1e-13
    z = np.eye(600) + 0.3 * rng.standard_normal((600, 600)) / np.sqrt(600)
    d, left, right = mm.blochMessiahVecs(z)
    assert _rel(left @ np.diag(d) @ right, z) < 1e-12
    assert _rel(np.sort(d), np.sort(np.linalg.svd(z, compute_uv=False))) < 1e-13


@pytest.mark.parametrize("phi,tol", [(0.1, 1e-3), (0.4, 1.5e-2)])
def test_squeezing_known_answer(nlm, mm, phi, tol):
    """The reference's Shirasaki notebook (tests/08 - Shirasaki.py): a Gaussian pulse in a Chi3 fibre
    over a nonlinear phase phi, squeezed below shot noise as Haus's formula
    1 + 2 phi^2 / sqrt 3 - (2 phi^3 / sqrt 3 + sqrt 2 phi) / sqrt(1 + phi^2) predicts for small phi,
    through the engine's Green's function and the GPU consumers (quadrature matrix, covariance,
    local-oscillator squeezing)."""
    m = nlm.Chi3(relativeLength=phi, nlLength=1, beta2=-1, pulseType=0, tPrecision=512, zPrecision=200)
    C, S = m.computeGreensFunction()
    Z = mm.calcQuadratureGreens(C, S)
    cov = mm.calcCovarianceMtx(Z, tol=1e-2)
    v = np.real(np.asarray(mm.calcLOSqueezing(cov, m.pumpTime[-1], tol=1e-2)))
    haus = 1 + 2 * phi ** 2 / np.sqrt(3) - (2 * phi ** 3 / np.sqrt(3) + np.sqrt(2) * phi) / np.sqrt(1 + phi ** 2)
    assert abs(v[0] - haus) < tol * haus
    assert v[1] > 1.0                                   # the conjugate quadrature is anti-squeezed
