"""The allocation-free preconditioner entry point.

sgfem_precondition_device_static serves callers that cannot allocate device
memory when they apply the preconditioner (a Julia process whose CUDA.jl pool
owns the GPU, a fixed device-memory budget, a loop that must not pay for
cudaMalloc's synchronisation).  It must give the same result as the ordinary
entry point sgfem_precondition, call after call, and it must refuse vectors
larger than its static scratch array.  This file is collected last so that a
failure here cannot hide the results of the other GPU tests."""
import numpy as np
import pytest

from tests.problems import build, config1_like

pytestmark = pytest.mark.gpu

STATIC_BYTES = 32 * 1024 * 1024  # SGFEM_STATIC_SCRATCH_BYTES in include/sgfem.h


@pytest.fixture(scope="module")
def setup(built_pkg):
    torch = pytest.importorskip("torch")
    p = config1_like()
    op = p.pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    assert op.has_lattice
    yield p, op, torch
    op.close()


@pytest.mark.parametrize("precision", ["FP64", "FP32"])
def test_static_matches_allocating_entry_point(setup, precision):
    p, op, torch = setup
    prec = getattr(p.pkg, precision)
    ctx = op.ctx
    n_dev, ld = ctx.device_layout()
    dtype = torch.float64 if precision == "FP64" else torch.float32
    assert n_dev * ld * dtype.itemsize <= STATIC_BYTES
    rng = np.random.default_rng(21)
    tol = 1e-12 if precision == "FP64" else 1e-6
    for call in range(2):  # two calls in a row share (and reuse) the static array
        b = rng.standard_normal(p.n * p.P)
        for mu in range(p.P):
            b[mu * p.n + p.bdofs] = 0.0
        ref = op.ldiv(b, p.pkg.PREC_LATTICE, prec)
        r_dev = torch.empty(n_dev * ld, dtype=dtype, device="cuda:0")
        z_dev = torch.full((n_dev * ld,), float("nan"), dtype=dtype, device="cuda:0")
        # the library works on its own stream: torch's fill must be done first
        torch.cuda.synchronize()
        ctx.to_device_layout(b, r_dev.data_ptr(), prec)
        ctx.precondition_device_static(r_dev.data_ptr(), z_dev.data_ptr(), prec)
        z = np.empty(p.n * p.P)
        ctx.from_device_layout(z_dev.data_ptr(), z, prec)
        assert np.all(np.isfinite(z))
        assert np.linalg.norm(z - ref) <= tol * np.linalg.norm(ref)


def test_static_rejects_vectors_beyond_the_maximum(built_pkg):
    torch = pytest.importorskip("torch")
    import __graft_entry__ as ge
    pkg = ge.load_package()
    C = pkg.StochasticCoefficientCosinus(tau=0.9, start=1, decay=2, mean=1.0, maxm=150)
    p = build(256, 1, 6, pkg.top_weight_multiindices(6, 150, C.decay_factors))
    op = pkg.SGOperator(p.V, p.TB, p.Kall, device=0)
    n_dev, ld = op.ctx.device_layout()
    assert n_dev * ld * 8 > STATIC_BYTES
    r = torch.zeros(n_dev * ld, dtype=torch.float64, device="cuda:0")
    z = torch.zeros_like(r)
    torch.cuda.synchronize()
    with pytest.raises(pkg.SGError) as e:
        op.ctx.precondition_device_static(r.data_ptr(), z.data_ptr(), pkg.FP64)
    assert e.value.code == 1 and "static maximum" in str(e.value)
    op.close()
