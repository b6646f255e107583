"""The algorithmic work model behind bench.py's roofline: each weight-adjusted
mass solve counts the cheaper of the reference's two sum-factorised
applications of V and the dense n_p x n_p product the kernels run, its
operator's bytes are counted where a phase applies it, bases without a
Vandermonde (nodal, diagonal mass matrix) count no mass-solve work, and the
per-element figures of the benchmark configurations stay pinned."""
import pytest


def _host(pkg, name, p):
    s = pkg.setups
    if name == "tgv":
        return s.tgv_tet(cells=1, p=p, lf=True).host_arrays()
    if name == "vortex":
        return s.vortex_tri(cells=2, p=p).host_arrays()
    return s.advection_tri(cells=2, p=p).host_arrays()


@pytest.mark.parametrize("name,p", [("tgv", 2), ("tgv", 4), ("tgv", 5), ("vortex", 4), ("advection", 4)])
def test_mass_solve_counts_the_cheaper_form(pkg, name, p):
    fm = pkg.flops_model
    host = _host(pkg, name, p)
    ra = host.sd.reference_approximation
    mf = fm.mass_solve_flops(ra)
    assert mf == min(2 * fm.vdm_flops(ra), 2.0 * ra.N_p * ra.N_p)
    assert mf < 2 * fm.vdm_flops(ra)          # the dense product is the cheaper one here
    w = fm.model(host)
    assert w.flops_A > 0 and w.flops_B > 0 and w.bytes_stage == 8.0 * 5 * host.N_p * host.N_c


def test_nodal_basis_has_no_mass_solve_work(pkg):
    fm = pkg.flops_model
    host = pkg.setups.tgv_tet(cells=1, p=3, approx="NodalTensor", lf=True).host_arrays()
    ra = host.sd.reference_approximation
    assert ra.V is None
    assert fm.mass_solve_flops(ra) == 0.0


def test_benchmark_work_per_element_is_pinned(pkg):
    """24,576-tet Taylor-Green benchmark (ModalTensor(4), FD, EC + LF): the
    per-element numbers that bench.py's roofline divides by."""
    w = pkg.flops_model.model(_host(pkg, "tgv", 4))
    assert w.flops_A == 67675.0
    assert w.flops_B == 367825.0
    assert w.bytes_A == 22200.0
    assert w.bytes_B == 52200.0
