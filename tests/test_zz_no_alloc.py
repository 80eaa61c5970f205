"""The allocation-free re-assembly, checked against the ordinary entry point.

fq_reassemble_noalloc serves callers that cannot let the library allocate
device memory (a host that owns all of it through its own arena, or a loop
where an allocation would synchronise the device); its element buffer is a
static device array. This file is collected last so that a run stopping at the
first failure has already run every other test; it also passes alone in a
fresh process (it makes its own context and mesh).
"""
import numpy as np
import pytest

import formoniq_gb300 as fq

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision,tol", [(fq.FQ_FP64, 1e-12), (fq.FQ_FP64_IEEE, 1e-12), (fq.FQ_FP32, 1e-6)])
def test_noalloc_reassembly_matches_fq_assemble_on_two_calls(precision, tol):
    """Every precision mode (float-float, IEEE double, FP32 values into a
    float32 buffer), two calls in a row on new lengths, each against the
    ordinary entry point in the same precision."""
    import torch

    ctx = fq.Context(0)
    mesh = fq.Mesh.kuhn_cube(ctx, 3, 6)
    wc = fq.WhitneyComplex(mesh, precision=precision)
    dtype = torch.float32 if precision == fq.FQ_FP32 else torch.float64
    for call, seed in enumerate((3, 4)):
        mesh.kuhn_lengths(jitter=0.1, seed=seed)
        for name, k in (("mass", 1), ("dif_both", 2), ("dif_test", 2)):
            m = getattr(wc, name)(k)  # the existing entry point on the new lengths
            expect = m.to_scipy().data.astype(np.float64)
            out = torch.full((m.nnz,), float("nan"), dtype=dtype, device="cuda")
            torch.cuda.synchronize()
            m.reassemble_noalloc(mesh, out.data_ptr())
            got = out.cpu().numpy().astype(np.float64)
            err = np.linalg.norm(got - expect) / np.linalg.norm(expect)
            assert err <= tol, (precision, call, name, k, err)
    ctx.close()


def test_noalloc_rejects_a_mesh_beyond_the_static_maximum():
    ctx = fq.Context(0)
    mesh = fq.Mesh.kuhn_cube(ctx, 3, 40)  # 384,000 cells x 21 entries x 8 B > 32 MiB
    mesh.kuhn_lengths(jitter=0.1, seed=1)
    m = fq.WhitneyComplex(mesh).mass(1)
    import torch

    out = torch.empty(m.nnz, dtype=torch.float64, device="cuda")
    with pytest.raises(fq.FqError) as e:
        m.reassemble_noalloc(mesh, out.data_ptr())
    assert e.value.name == "FQ_INVALID_ARG" and "static maximum" in str(e.value)
    ctx.close()
