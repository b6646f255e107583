"""Small seeded parity cases covering every form / law / element / basis
combination of the hot path.  Each case returns (HostArrays, u) with u the
configuration's initial state plus a seeded 1e-3 perturbation of every
modal coefficient (the same construction as the benchmark inputs)."""
import math

import numpy as np

import __graft_entry__

PKG = __graft_entry__.load_package()
S = PKG.solver
M = PKG.mesh
R = PKG.reference
setups = PKG.setups

SEED = 20261203


def _disc(approx, shape, p, cells, L, warp, metrics):
    ra = R.reference_approximation(approx, shape, p, mapping_degree=p)
    d = 2 if shape == "Tri" else 3
    mesh = M.uniform_periodic_mesh(ra, ((0.0, L),) * d, (cells,) * d)
    mesh = M.warp_mesh(mesh, ra, "Chan", warp, (L,) * d)
    return M.spatial_discretization(mesh, ra, metrics=metrics)


def _disc_multi(approx, shape, p, cells, L, warp, metrics):
    """ModalMulti / NodalMulti with the collapsed Gauss rules of setups.multi_rules."""
    d = 2 if shape == "Tri" else 3
    return setups._disc(approx, shape, p, ((0.0, L),) * d, (cells,) * d, "Chan", warp, metrics)


def make(name):
    seed = SEED + sum(map(ord, name))
    if name.startswith("multi_"):
        # multidimensional (dense-operator) approximations
        approx = "NodalMulti" if "nodal" in name else "ModalMulti"
        if "_adv_" in name:
            sd = _disc_multi(approx, "Tri", 4, 4, 1.0, 0.1, "Exact")
            law = S.LinearAdvectionEquation((1.0, 1.0))
            ic = S.InitialDataSine(1.0, (2 * math.pi, 2 * math.pi))
            form = S.StandardForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux())
            if "fd" in name:
                form = S.FluxDifferencingForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux())
        elif "_tri" in name:
            vort = setups.vortex_tri(cells=2, p=2)
            sd = _disc_multi(approx, "Tri", 3, 8, 10.0, 0.1, "ChanWilcox")
            law, ic = vort.law, vort.initial_data
            nflux = S.EntropyConservativeNumericalFlux() if "ec" in name else S.LaxFriedrichsNumericalFlux()
            form = S.FluxDifferencingForm(inviscid_numerical_flux=nflux)
            if "std" in name:
                form = S.StandardForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux())
        else:
            tgv = setups.tgv_tet(cells=1, p=2)
            sd = _disc_multi(approx, "Tet", 3, 2, 2 * math.pi, 0.05, "ChanWilcox")
            law, ic = tgv.law, tgv.initial_data
            nflux = S.EntropyConservativeNumericalFlux() if "ec" in name else S.LaxFriedrichsNumericalFlux()
            form = S.FluxDifferencingForm(inviscid_numerical_flux=nflux)
        host = S.HostArrays(law, sd, form)
        u0 = S.initialize(ic, sd)
        return host, setups.perturbed(u0, seed, 1.0e-3)
    if name.startswith("adv_tri"):
        approx = "NodalTensor" if "nodal" in name else "ModalTensor"
        sd = _disc(approx, "Tri", 4, 4, 1.0, 0.1, "Exact")
        law = S.LinearAdvectionEquation((1.0, 1.0))
        lam = 0.0 if "central" in name else 1.0
        form = S.StandardForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux(lam))
        if "fd" in name:
            form = S.FluxDifferencingForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux())
        ic = S.InitialDataSine(1.0, (2 * math.pi, 2 * math.pi))
    elif name.startswith("adv_tet"):
        sd = _disc("ModalTensor", "Tet", 3, 2, 1.0, 0.05, "Exact")
        law = S.LinearAdvectionEquation((1.0, 0.5, -0.25))
        form = S.StandardForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux())
        if "fd" in name:
            form = S.FluxDifferencingForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux())

        class Ic:
            N_c = 1

            def evaluate(self, x, t=0.0):
                return (np.sin(2 * np.pi * x[0]) * np.cos(2 * np.pi * x[1]) + x[2] * 0 + 1.0)[..., None]
        ic = Ic()
    elif name.startswith("vortex_tri") or name.startswith("euler_tri"):
        approx = "NodalTensor" if "nodal" in name else "ModalTensor"
        pb = setups.vortex_tri(cells=8, p=3, approx=approx,
                               metrics="Exact" if "exact" in name else "ChanWilcox")
        sd, law, ic = pb.sd, pb.law, pb.initial_data
        nflux = S.EntropyConservativeNumericalFlux() if "ec" in name else S.LaxFriedrichsNumericalFlux()
        two = S.ConservativeFlux() if "cons2pt" in name else S.EntropyConservativeFlux()
        if "chandra" in name:
            two = S.ChandrashekarFlux()
        form = S.FluxDifferencingForm(inviscid_numerical_flux=nflux, two_point_flux=two)
        if name.startswith("euler_tri"):
            form = S.StandardForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux())
    elif name.startswith("tgv_tet") or name.startswith("euler_tet"):
        approx = "NodalTensor" if "nodal" in name else "ModalTensor"
        p = 6 if "p6" in name else (5 if "p5" in name else (2 if "p2" in name else (3 if "nodal" in name else 4)))
        if name.startswith("euler_tet"):
            p = 3
        pb = setups.tgv_tet(cells=2, p=p, approx=approx, lf="ec" not in name,
                            metrics="Exact" if "exact" in name else "ChanWilcox")
        sd, law, ic, form = pb.sd, pb.law, pb.initial_data, pb.form
        if "cons2pt" in name:
            form = S.FluxDifferencingForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux(),
                                          two_point_flux=S.ConservativeFlux())
        if "chandra" in name:
            nflux = S.EntropyConservativeNumericalFlux() if "ec" in name else S.LaxFriedrichsNumericalFlux()
            form = S.FluxDifferencingForm(inviscid_numerical_flux=nflux, two_point_flux=S.ChandrashekarFlux())
        if name.startswith("euler_tet"):
            form = S.StandardForm(inviscid_numerical_flux=S.LaxFriedrichsNumericalFlux())
    else:
        raise KeyError(name)
    host = S.HostArrays(law, sd, form)
    u0 = S.initialize(ic, sd)
    u = setups.perturbed(u0, seed, 1.0e-3)
    return host, u


NAMES = ["adv_tri_modal", "adv_tri_nodal", "adv_tri_central", "adv_tri_fd", "adv_tet_modal",
         "adv_tet_fd", "vortex_tri_modal", "vortex_tri_nodal", "vortex_tri_ec",
         "vortex_tri_cons2pt", "euler_tri_std", "tgv_tet_modal", "tgv_tet_ec", "tgv_tet_nodal",
         "tgv_tet_p5", "tgv_tet_p6", "tgv_tet_p2", "tgv_tet_cons2pt", "euler_tet_std",
         "vortex_tri_chandra", "tgv_tet_chandra", "vortex_tri_exact", "tgv_tet_exact",
         "tgv_tet_ec_exact", "tgv_tet_nodal_exact"]
# Euler FD meshes built with the reference's default exact metrics, which on
# curved tets do not preserve a free stream
EXACT_NAMES = ["vortex_tri_exact", "tgv_tet_exact", "tgv_tet_ec_exact", "tgv_tet_nodal_exact"]
# multidimensional (dense V, D, R) approximations: parity, adjoint and mixed cases
MULTI_NAMES = ["multi_adv_tri", "multi_adv_tri_nodal", "multi_adv_tri_fd", "multi_tri",
               "multi_tri_nodal", "multi_tri_std", "multi_tri_ec", "multi_tet", "multi_tet_ec",
               "multi_tet_nodal"]
