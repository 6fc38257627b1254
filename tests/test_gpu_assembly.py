"""GPU parity of getOPERATORS (Toeplitz, circulant, FFT of circulant), the
singular integrals and the excitations against the oracle and the reference's
golden DIRECTFN / cubature values."""
import numpy as np
import pytest

from oracle import vie_oracle as vo

pytestmark = pytest.mark.gpu
FREQ = 298e6


def relerr(a, b):
    return np.max(np.abs(np.asarray(a) - np.asarray(b))) / np.max(np.abs(b))


def test_directfn_matches_reference_golden(golden):
    """The device DIRECTFN (the default singular method) against the values of
    the reference's own C++ cores at Np_1D = 20 and 64: 1e-13 relative."""
    import marie_gb300 as mg

    for d in golden["directfn"]:
        ref = np.array(d["re"]) + 1j * np.array(d["im"])
        dev = mg.singular_integrals(d["ko"], d["dx"], np_1d=d["Np"])
        rel = np.abs(dev - ref) / np.abs(ref)
        assert rel.max() < 1e-13, (d["ko"], d["dx"], d["Np"], rel)
        if d["Np"] == 20:  # the default order
            assert np.array_equal(mg.singular_integrals(d["ko"], d["dx"]), dev)


def test_directfn_single_calls_match_reference_golden(golden):
    """Each DIRECTFN core through its gateway's vertex order (marie_directfn)
    on seeded random triangles, against the reference C++: 1e-12 relative."""
    import marie_gb300 as mg

    for c in golden["directfn_tri"]:
        v = mg.directfn(c["kind"], c["r"], c["ko"], c["Np"])
        ref = c["re"] + 1j * c["im"]
        assert abs(v - ref) / abs(ref) < 1e-12, (c["kind"], c["Np"], abs(v - ref) / abs(ref))


def test_converged_singular_integrals_match_oracle(golden):
    import marie_gb300 as mg

    for d in golden["directfn"][:4]:
        dev = mg.singular_integrals(d["ko"], d["dx"], method="CONVERGED")
        ora = vo.singular_integrals(d["ko"], d["dx"], method="CONVERGED")
        np.testing.assert_allclose(dev, ora, rtol=1e-13)


def test_singular_method_arguments():
    import marie_gb300 as mg

    r = vo.grid(4, 4, 4, 5e-3)
    with pytest.raises(ValueError):
        mg.getOPERATORS(r, FREQ, singular="DEMCEM")
    with pytest.raises(ValueError):
        mg.singular_integrals(6.2, 5e-3, method="DEMCEM")
    lib = mg.load()
    out = np.zeros(10)
    import ctypes as C

    assert lib.marie_singular_integrals_ex(6.2, 5e-3, b"E", 0, C.c_void_p(out.ctypes.data)) == mg._lib.MARIE_EINVAL
    assert lib.marie_singular_integrals_ex(6.2, 5e-3, b"D", 65, C.c_void_p(out.ctypes.data)) == mg._lib.MARIE_EINVAL


@pytest.mark.parametrize("shape,dx", [((8, 8, 8), 5e-3), ((12, 4, 8), 2e-3), ((6, 7, 5), 3e-3)])
def test_toeplitz_matches_oracle(shape, dx):
    import marie_gb300 as mg

    r = vo.grid(*shape, dx)
    ref = vo.getOPERATORS(r, FREQ, typ="T")
    out = mg.getOPERATORS(r, FREQ, "N", "T")
    assert relerr(out, ref) < 1e-12


@pytest.mark.parametrize("dx", [5e-3, 2e-3])
def test_default_operator_is_the_references(golden, dx):
    """getOPERATORS and Operator.assemble with default arguments against the
    oracle fed the reference's own DIRECTFN values (Np_1D = 20, from its C++
    cores): 1e-12.  The same through singular_values ('U')."""
    import marie_gb300 as mg

    d = [g for g in golden["directfn"] if g["dx"] == dx and g["Np"] == 20 and g["ko"] == golden["directfn"][0]["ko"]][0]
    sv = np.array(d["re"]) + 1j * np.array(d["im"])
    r = vo.grid(8, 8, 8, dx)
    ref = vo.getOPERATORS(r, FREQ, sing=sv)
    assert relerr(mg.getOPERATORS(r, FREQ), ref) < 1e-12
    assert relerr(mg.Operator.assemble(8, 8, 8, dx, FREQ).to_array(), ref) < 1e-12
    assert relerr(mg.getOPERATORS(r, FREQ, singular_values=sv), ref) < 1e-12
    assert relerr(mg.getOPERATORS(r, FREQ, "N", "T"), vo.getOPERATORS(r, FREQ, typ="T", sing=sv)) < 1e-12
    # the converged quadrature (opt-in) moves fN by about 6e-5 of its maximum
    conv = mg.getOPERATORS(r, FREQ, singular="CONVERGED")
    assert 1e-6 < relerr(conv, ref) < 2e-4


@pytest.mark.parametrize("shape", [(8, 8, 8), (12, 16, 4), (24, 8, 20)])
def test_circulant_and_fft_match_oracle(shape):
    import marie_gb300 as mg

    r = vo.grid(*shape, 5e-3)
    C = vo.getOPERATORS(r, FREQ, typ="C")
    F = vo.fft_operator(C)
    assert relerr(mg.getOPERATORS(r, FREQ, "N", "C"), C) < 1e-12
    assert relerr(mg.getOPERATORS(r, FREQ), F) < 1e-12
    op = mg.Operator.assemble(*shape, 5e-3, FREQ)
    assert relerr(op.to_array(), F) < 1e-12


def test_plane_wave_and_dipoles_match_oracle():
    import marie_gb300 as mg

    r = vo.grid(12, 8, 16, 4e-3)
    em = vo.EMconstants(FREQ)
    for k, Eo in (([0, 0, em["ko"]], [1, 0, 0]), ([em["ko"] / 2, 0, em["ko"] * 0.8], [0, 1j, 0.5])):
        Eref, Href = vo.PlaneWave_Excitation(r, k, em["omega_mu"], Eo)
        E, H = mg.PlaneWave_Excitation(r, k, em["omega_mu"], Eo)
        assert relerr(E, Eref) < 1e-13
        assert relerr(H, Href) < 1e-13
    pos = np.array([[0.15, 0, 0.01], [0, -0.15, -0.05], [-0.1, 0.1, 0.0]])
    Jd = np.array([[0, 0, 1], [0, 0, 1], [0.3, 0, 1j]], complex)
    Eref = vo.Dipole_Excitation(r, em["ko"], Jd, pos)
    E = mg.Dipole_Excitation(r, em["ko"], Jd, pos)
    assert relerr(E, Eref) < 1e-12


def test_e_field_nop_matches_oracle():
    import marie_gb300 as mg

    L, M, N = 8, 12, 8
    rng = np.random.default_rng(0)
    r = vo.grid(L, M, N, 5e-3)
    fN = vo.getOPERATORS(r, FREQ)
    J = np.asfortranarray(rng.standard_normal((L, M, N, 3)) + 1j * rng.standard_normal((L, M, N, 3)))
    Ei = np.asfortranarray(rng.standard_normal((L, M, N, 3)) + 0j)
    ref = vo.E_field_Nop(J, fN, 1.25e-7, FREQ, Ei)
    out = mg.E_field_Nop(J, mg.Operator.from_array(fN), 1.25e-7, FREQ, Ei)
    assert relerr(out, ref) < 1e-12
