"""The throughput form of the oracle's tangent and heat vmults (oracle/oracle_fast.hpp,
timed as the CPU baseline) gives the oracle's vmult (mf_nh_operator.h:545-625)
to round-off: every degree 1-6, every caching variant, every lane count,
on meshes whose colours leave partly filled cell batches and with a clamped
face (constrained DoFs read as zero, identity rows)."""
import numpy as np
import pytest

import oracle as O
import workloads as W

ANISO = dict(rep=(3, 1, 1), length=(3.0, 1.0, 0.7))


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("caching", ["scalar_referential", "tensor2", "tensor4", "tensor4_ns"])
@pytest.mark.parametrize("lanes", [2, 4, 8])
def test_fast_form_matches_oracle(degree, caching, lanes):
    mat = O.material(0.5e6, 0.4, 1000.0, 0.01)
    for n_ref in (0, 1):
        spec = W.cantilever(degree, n_ref, **ANISO)
        u = W.smooth_displacement(degree, n_ref, spec["rep"], spec["lo"], spec["hi"], seed=3)
        om = W.to_oracle_mesh(O, spec)
        x = W.uniform_vector(len(u), 12)
        ref = O.nh_vmult(om, n_ref, mat, caching, u, x)
        got, secs = O.nh_vmult_fast_timed(om, n_ref, mat, caching, u, x, 2, lanes=lanes)
        assert rel(got, ref) < 1e-13, (n_ref, rel(got, ref))
        assert secs > 0.0


def test_fast_form_rejects_what_it_does_not_cover():
    spec = W.cantilever(2, 0, **ANISO)
    u = W.smooth_displacement(2, 0, spec["rep"], spec["lo"], spec["hi"], seed=3)
    om = W.to_oracle_mesh(O, spec)
    x = W.uniform_vector(len(u), 12)
    with pytest.raises(RuntimeError):
        O.nh_vmult_fast_timed(om, 0, O.material(0.5e6, 0.4, 1000.0, 0.01, formulation=0),
                              "tensor4_ns", u, x, 1)
    with pytest.raises(RuntimeError):
        O.nh_vmult_fast_timed(om, 0, O.material(0.5e6, 0.4, 1000.0, 0.01), "tensor4_ns", u, x, 1,
                              lanes=3)


@pytest.mark.parametrize("degree", [1, 2, 3, 4, 5, 6])
@pytest.mark.parametrize("lanes", [2, 4, 8])
def test_fast_heat_matches_oracle(degree, lanes):
    """The heat operator M + k dt K (heat_transfer.h:236-250) in the same
    form, with a Dirichlet face, to round-off."""
    for n_ref in (0, 1):
        spec = W.unit_cube_heat(degree, n_ref, rep=(3, 1, 1))
        spec["hi"] = (1.0, 0.6, 0.45)
        om = W.to_oracle_mesh(O, spec)
        x = W.uniform_vector(W.n_dofs(spec, 1), 13)
        ref = O.heat_vmult(om, n_ref, 0.1, x)
        got, secs = O.heat_vmult_fast_timed(om, n_ref, 0.1, x, 2, lanes=lanes)
        assert rel(got, ref) < 1e-13, (n_ref, rel(got, ref))
        assert secs > 0.0
