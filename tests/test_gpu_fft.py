"""FP64 stencil sums by FFT (TGPU_FILL_FFT): the accurate fill's long 3-D sums (the attraction stencil) as
FFT convolutions, the short ones (theta, delta) as float-float sums.

- At the fixture states of the 3-D reference cases (FMT1+WCA rough wall, FMT2/FMT4 rough walls) the
  TGPU_FILL_FFT residual with every stencil sum taken by FFT (forward multi-output delta sums, transposed
  delta and theta sums, attraction) equals the reference's to the 1e-12 of the FP64 parity tests;
- on the 64^3 configuration-2 problem (default choice: the attraction sum by FFT) and with every sum by FFT
  it equals the direct FP64 fill to 5e-12 at the initial state (the FFT's rounding, ~eps log2 of the box
  times the sums' scale, against the direct sums' own ~1e-12);
- a TGPU_FILL_MIXED_FFT Newton solve reaches ||R||_2 <= 1e-8, its residual re-evaluated by the direct
  FP64 fill is below 1e-8 too, and its density equals the FP64 solve's to 1e-9;
- with every FP32 sum forced onto FP32 FFTs (tgpu_set_fft32_policy 1) the Schur product equals the FP64 one to
  1e-5, its nonlocal part (S v2 less the local v2 / rho) too, and J v to 1e-5 (relative to their max norms), an FP32 fill equals the FP64 fill to 1e-4, and the mixed
  solve still reaches the FP64 solve's density to 1e-9; with the direct kernels forced (policy 0) the products
  are the slab / tensor-core ones;
- FP32 Schur products whose every sum is an FP32 FFT keep their sums, channels and transposed sums in FP32 storage;
  with the timed choices (policy -1) the first product makes the choices in FP64 storage, the next ones run in
  FP32 storage and equal it to 1e-6 (the same FP32 sums; only the last sum A21 y rounds in FP32);
- TGPU_FP64_FFT products (J v and the Schur product with the sums of TGPU_FILL_FFT) equal the reference's
  assembled products on the 3-D fixtures to 1e-12 (every sum by FFT) and the direct FP64 products at 64^3 to 1e-11.
"""
import numpy as np
import pytest

from goldens import RESID_ATOL, load

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["fmt1_wca_3d", "rough3d_fmt2", "rough3d_fmt4"])
def test_fft_fill_matches_reference_fixture(name):
    from tramonto_gb300 import native
    z, p = load(name)
    s = native.Solver(p)
    s.set_fill_arithmetic(native.FILL_FFT)
    s.set_fft_threshold(0)   # every stencil by FFT: the multi-output delta sums and the transposed sums too
    for k in range(len(z["states"])):
        R = s.fill(z[f"x{k}"], mode=1)
        err = np.abs(R - z[f"R{k}"]).max()
        print(name, "state", k, "max |R_fft - R_ref|", err)
        assert err <= RESID_ATOL, (name, k, err)
    s.close()


def test_fft_fill_matches_fp64_fill():
    from tramonto_gb300 import native, setup
    p, _ = setup.config2(n=64)
    s = native.Solver(p)
    x = setup.initial_state(s, p)
    R64 = s.fill(x, mode=1)
    s.set_fill_arithmetic(native.FILL_FFT)
    for thr in (-1, 0):
        s.set_fft_threshold(thr)
        Rfft = s.fill(x, mode=1)
        err = np.abs(Rfft - R64).max()
        print("64^3 threshold", thr, ": max |R_fft - R_fp64|", err, "max |R|", np.abs(R64).max(),
              "||R_fft - R_fp64||_2", np.linalg.norm(Rfft - R64))
        assert err <= 5e-12
    s.close()


def test_mixed_fft_newton_solve():
    from tramonto_gb300 import native, setup
    p, _ = setup.config2(n=40)
    s = native.Solver(p)
    x0 = setup.initial_state(s, p)
    x64, _, _, _ = s.newton_solve(x0, resid_tol=1e-8, lin_tol=1e-10)
    s.set_precision(native.FP16TC)
    s.set_fill_arithmetic(native.FILL_MIXED_FFT, switch_norm=0.1)
    xf, it, rn, li = s.newton_solve(x0, resid_tol=1e-8, lin_tol=1e-6)
    assert rn <= 1e-8
    s.set_fill_arithmetic(native.FILL_FP64)
    r64 = np.linalg.norm(s.fill(xf, mode=1))
    print("mixed-FFT solve:", it, "iterations, ||R||_2", rn, "re-evaluated in FP64", r64)
    assert r64 <= 1e-8
    assert np.abs(xf[p.first_rho] - x64[p.first_rho]).max() <= 1e-9
    s.close()


@pytest.mark.parametrize("policy", [1, 0])
def test_fp32_fft_products(policy):
    from tramonto_gb300 import native, setup
    from goldens import rel_err
    p, _ = setup.config2(n=40)
    s = native.Solver(p)
    x0 = setup.initial_state(s, p)
    x64, _, _, _ = s.newton_solve(x0, resid_tol=1e-8, lin_tol=1e-10)
    s.fill(x64)
    rng = np.random.default_rng(4)
    v2 = rng.standard_normal((p.ncomp, p.nnodes))
    v = rng.standard_normal((p.nunk, p.nnodes))
    S64, J64 = s.schur(v2), s.jv(v)
    s.set_precision(native.FP16TC)
    s.set_fft32_policy(policy)
    S32, J32 = s.schur(v2), s.jv(v)
    # the nonlocal part of S v2 (the local A22 v2 = v2 / rho on live rows dominates the max norm near the wall)
    rho = x64[p.first_rho:p.first_rho + p.ncomp]
    live = (np.asarray(p.zero_density).reshape(rho.shape) == 0) & (np.asarray(p.vext).reshape(rho.shape) < p.vext_max)
    local = np.where(live, v2 / np.where(live, rho, 1.0), v2)
    nl64, nl32 = S64 - local, S32 - local
    print("policy", policy, "Schur rel", rel_err(S32, S64), "nonlocal part rel", rel_err(nl32, nl64),
          "Jv rel", rel_err(J32, J64))
    assert rel_err(S32, S64) <= 1e-5 and rel_err(J32, J64) <= 1e-5
    assert rel_err(nl32, nl64) <= 1e-5
    s.set_fill_arithmetic(native.FILL_FP32)
    R32 = s.fill(x64, mode=1)
    s.set_fill_arithmetic(native.FILL_FP64)
    R64 = s.fill(x64, mode=1)
    assert np.abs(R32 - R64).max() <= 1e-4 * max(1.0, np.abs(R64).max())
    s.set_fill_arithmetic(native.FILL_MIXED_FFT, switch_norm=0.1)
    xf, it, rn, _ = s.newton_solve(x0, resid_tol=1e-8, lin_tol=1e-6)
    assert rn <= 1e-8
    assert np.abs(xf[p.first_rho] - x64[p.first_rho]).max() <= 1e-9
    s.close()


@pytest.mark.parametrize("name", ["fmt1_wca_3d", "rough3d_fmt2", "rough3d_fmt4"])
def test_fp64_fft_products_match_reference_fixture(name):
    """TGPU_FP64_FFT products (every 3-D sum by FP64 FFT with threshold 0) against the reference's assembled
    J v and Schur product, to the 1e-12 of the FP64 parity tests."""
    from tramonto_gb300 import native
    from goldens import PROD_RTOL, probe, rel_err
    z, p = load(name)
    s = native.Solver(p)
    s.set_precision(native.FP64_FFT)
    s.set_fft_threshold(0)
    N = p.nunk * p.nnodes
    for k in range(len(z["states"])):
        x = z[f"x{k}"]
        s.fill(x)
        Jv = s.jv(probe(N, 0).reshape(x.shape))
        S = s.schur(probe(p.ncomp * p.nnodes, 2).reshape(p.ncomp, p.nnodes))
        print(name, k, "Jv rel", rel_err(Jv, z[f"Jv{k}"]), "Sv rel", rel_err(S, z[f"schur_Sv{k}"]))
        assert rel_err(Jv, z[f"Jv{k}"]) <= PROD_RTOL
        assert rel_err(S, z[f"schur_Sv{k}"]) <= PROD_RTOL
    s.close()


def test_fp64_fft_products_match_fp64_products():
    """At 64^3 (default choice: the attraction sum by FP64 FFT, theta and delta in float-float) the Schur
    product and J v equal the direct FP64 ones to 1e-11 of their max norms."""
    from tramonto_gb300 import native, setup
    from goldens import rel_err
    p, _ = setup.config2(n=64)
    s = native.Solver(p)
    x = setup.initial_state(s, p)
    s.fill(x)
    rng = np.random.default_rng(8)
    v2 = rng.standard_normal((p.ncomp, p.nnodes))
    v = rng.standard_normal((p.nunk, p.nnodes))
    S64, J64 = s.schur(v2), s.jv(v)
    s.set_precision(native.FP64_FFT)
    S, J = s.schur(v2), s.jv(v)
    print("64^3 FP64-FFT products: Schur rel", rel_err(S, S64), "Jv rel", rel_err(J, J64))
    assert rel_err(S, S64) <= 1e-11 and rel_err(J, J64) <= 1e-11
    s.close()


def test_fft_sums_follow_a_moved_bulk_state():
    """After tgpu_set_bulk_state (the continuation in the chemical potential) the FFT sums read the new bulk values
    at the bulk boundary as the direct sums do: FP64-FFT fill = direct FP64 fill to 5e-12, FP32 fill to 1e-4."""
    from tramonto_gb300 import native, setup
    p, _ = setup.config2(n=40)
    s = native.Solver(p)
    x = setup.initial_state(s, p, max_enhancement=1.0)
    s.set_bulk([0.66])
    R64 = s.fill(x, mode=1)
    s.set_fill_arithmetic(native.FILL_FFT)
    Rf = s.fill(x, mode=1)
    s.set_fill_arithmetic(native.FILL_FP32)
    R32 = s.fill(x, mode=1)
    print("moved bulk: |R_fft - R_fp64|", np.abs(Rf - R64).max(), "|R_fp32 - R_fp64|", np.abs(R32 - R64).max())
    assert np.abs(Rf - R64).max() <= 5e-12
    assert np.abs(R32 - R64).max() <= 1e-4 * max(1.0, np.abs(R64).max())
    s.close()


def test_fp32_storage_schur_product_equals_the_fp64_storage_one():
    from tramonto_gb300 import native, setup
    from goldens import rel_err
    p, _ = setup.config2(n=40)
    s = native.Solver(p)
    x0 = setup.initial_state(s, p)
    s.fill(x0)
    rng = np.random.default_rng(11)
    v2 = rng.standard_normal((p.ncomp, p.nnodes))
    S64 = s.schur(v2)
    s.set_precision(native.FP32)
    first = s.schur(v2)     # makes the timed FFT / direct choices (FP64 storage)
    again = s.schur(v2)     # FP32 storage when every sum took the FFT
    print("first vs again", rel_err(again, first), "vs FP64", rel_err(again, S64))
    assert rel_err(again, first) <= 1e-6
    assert rel_err(again, S64) <= 1e-5
    s.close()


@pytest.mark.parametrize("n", [96, 128])
def test_fp32_fft_codelet_lengths(n):
    """The compile-time codelets of the FP32 and FP64 passes (y/z lengths 96 and 128, x lengths 150 and 180 at 96^3
    and 128^3): with every FP32 sum an FFT the Schur product's nonlocal part and J v equal the FP64 products to 1e-5
    of their max norms, the FP32 fill the FP64 fill to 1e-4, and the FP64 FFT fill (every stencil by FFT) the direct
    FP64 fill to 5e-12, as at 64^3."""
    from tramonto_gb300 import native, setup
    from goldens import rel_err
    p, _ = setup.config2(n=n)
    s = native.Solver(p)
    x = setup.initial_state(s, p)
    s.fill(x)
    rng = np.random.default_rng(n)
    v2 = rng.standard_normal((p.ncomp, p.nnodes))
    v = rng.standard_normal((p.nunk, p.nnodes))
    S64, J64 = s.schur(v2), s.jv(v)
    s.set_precision(native.FP32)
    s.set_fft32_policy(1)
    S32, J32 = s.schur(v2), s.jv(v)
    rho = x[p.first_rho:p.first_rho + p.ncomp]
    live = (np.asarray(p.zero_density).reshape(rho.shape) == 0) & (np.asarray(p.vext).reshape(rho.shape) < p.vext_max)
    local = np.where(live, v2 / np.where(live, rho, 1.0), v2)
    print(n, "nonlocal Schur rel", rel_err(S32 - local, S64 - local), "Jv rel", rel_err(J32, J64))
    assert rel_err(S32 - local, S64 - local) <= 1e-5 and rel_err(J32, J64) <= 1e-5
    s.set_fill_arithmetic(native.FILL_FP32)
    R32 = s.fill(x, mode=1)
    s.set_fill_arithmetic(native.FILL_FP64)
    R64 = s.fill(x, mode=1)
    assert np.abs(R32 - R64).max() <= 1e-4 * max(1.0, np.abs(R64).max())
    s.set_fill_arithmetic(native.FILL_FFT)
    s.set_fft_threshold(0)
    Rfft = s.fill(x, mode=1)
    print(n, "FP64 FFT fill: max |R_fft - R_fp64|", np.abs(Rfft - R64).max())
    assert np.abs(Rfft - R64).max() <= 5e-12
    s.close()


def test_pass_timer_counts_the_fp32_pass_launches():
    """tgpu_pass_timer_begin/_end: over one FP32 Schur product with every sum an FFT it sees the y/z pass launches
    (two per transform batch), their summed duration, and per transform at least the half spectrum written and read
    once (8 bytes per complex point each way)."""
    from tramonto_gb300 import native, setup
    p, _ = setup.config2(n=40)
    s = native.Solver(p)
    x = setup.initial_state(s, p)
    s.fill(x)
    s.set_precision(native.FP32)
    s.set_fft32_policy(1)
    v2 = np.random.default_rng(2).standard_normal((p.ncomp, p.nnodes))
    s.schur(v2)
    s.pass_timer_begin()
    s.schur(v2)
    launches, ms, nbytes, transforms = s.pass_timer_end()
    _, nh, _ = s.time_fft_pass(native.FP32, 1, reps=1)
    print("launches", launches, "ms", ms, "bytes", nbytes, "transforms", transforms)
    assert launches > 0 and launches % 2 == 0 and ms > 0.0
    assert transforms >= launches and nbytes >= transforms * 2 * 8 * nh
    assert s.pass_timer_end()[0] == 0          # the timer is off and empty after end
    s.close()
