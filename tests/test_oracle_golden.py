"""The oracle against the reference's own golden regression outputs (CPU only).

Every case of the reference's test list whose features, optimiser and analysis the hot
path covers is run through the reference's program flow on the FP64 oracle and compared
with the reference program's outputs at the reference test driver's tolerance."""

import numpy as np
import pytest

import golden_cases as G
import oracle as O


class OracleBackend:
    acsf = staticmethod(O.acsf)
    zscore_stats = staticmethod(O.zscore_stats)
    zscore_apply = staticmethod(O.zscore_apply)
    predict = staticmethod(O.predict)
    jacobian = staticmethod(O.jacobian)
    forces = staticmethod(O.forces)
    train_gradients = staticmethod(O.train_gradients)
    update_prepare = staticmethod(O.update_prepare)
    ranlux = staticmethod(lambda seed: O.Ranlux(seed))
    sd = staticmethod(lambda x0, tol, md, lr: O.SteepestDescent(x0, tol, md, lr))
    lbfgs = staticmethod(lambda x0, tol, mi, ma, mem, lm, qn: O.Lbfgs(x0, tol, mi, ma, mem, lm, qn))
    cg = staticmethod(lambda x0, tol, ma: O.ConjGrad(x0, tol, ma))
    fire = staticmethod(lambda x0, tol, ma: O.Fire(x0, tol, ma))


@pytest.mark.parametrize("name", G.case_names())
def test_oracle_matches_reference_outputs(name):
    case = G.load_case(name)
    if case.settings["mode"] == "train":
        zprec, params = G.run_training(case, OracleBackend)
        out = case.net("out_")
        np.testing.assert_allclose(params, out["params"], rtol=G.RTOL, atol=G.ATOL)
        if zprec is not None and out["zprec"] is not None:
            np.testing.assert_allclose(zprec, out["zprec"], rtol=G.RTOL, atol=G.ATOL)
    else:
        pred, forces = G.run_prediction(case, OracleBackend)
        np.testing.assert_allclose(pred, case.arrays["out_rawpredictions"], rtol=G.RTOL,
                                   atol=G.ATOL)
        if forces is not None:
            np.testing.assert_allclose(forces.reshape(forces.shape[0], -1),
                                       case.arrays["out_forces"], rtol=G.RTOL, atol=G.ATOL)


def test_acsf_modes_agree():
    """Per-(atom, function) neighbour rebuild (the reference's loop) and one filtered list
    per atom give identical features."""
    case = G.load_case("analysis/derivatives/analytical/singleTarget/speciesResolved/raw")
    g = case.net("in_")["gfuncs"]
    a = O.acsf(case.ds, g, mode=0)
    b = O.acsf(case.ds, g, mode=1)
    assert np.array_equal(a, b)


def test_ranlux_threads_deterministic():
    case = G.load_case("analysis/derivatives/analytical/singleTarget/speciesResolved/raw")
    g = case.net("in_")["gfuncs"]
    a = O.acsf(case.ds, g, mode=1, nthreads=1)
    b = O.acsf(case.ds, g, mode=1, nthreads=3)
    assert np.array_equal(a, b)
