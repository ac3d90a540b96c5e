"""Searches on the GPU: SearchStep against the reference's own random-search
kernel (golden fixture), random search and second-order random search
against the oracle with the same counter-based draws."""
import os

import numpy as np
import pytest
import torch

from oracle import OracleModel
from pycompute_gb300 import RandomSearch, SearchStep, SecondOrderRandomSearch, parity, synth

pytestmark = pytest.mark.gpu
DEV = "cuda:0"
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def _t(a):
    return torch.from_numpy(np.ascontiguousarray(a)).to(DEV)


def test_search_step_matches_reference_golden():
    z = np.load(os.path.join(GOLD, "ivim21_search.npz"))
    N = z["p"].shape[1]
    ss = SearchStep(synth.IVIM_EXPR, synth.IVIM_PARS, ["b"], 21, torch.float32)
    lbv = np.zeros(4, np.float32)
    ubv = np.ones(4, np.float32)
    ss.setup(_t(z["protocol"]), _t(z["data"]), _t(lbv), _t(ubv))
    f = torch.zeros(N, device=DEV)
    bp, bf = _t(z["best_p_in"]), _t(z["best_f_in"])
    ss.run(f, bf, _t(z["p"]), bp)
    torch.cuda.synchronize()
    np.testing.assert_allclose(f.cpu().numpy(), z["f"], rtol=2e-6)
    np.testing.assert_allclose(bf.cpu().numpy(), z["best_f"], rtol=2e-6)
    np.testing.assert_array_equal(bp.cpu().numpy(), z["best_p"])


@pytest.fixture(scope="module")
def ivim_data():
    w = synth.ivim()
    true, data, init, lb, ub, prot = w.generate(4096, seed=21)
    return w, data, lb, ub, prot


def test_random_search_matches_oracle(ivim_data):
    w, data, lb, ub, prot = ivim_data
    rs = RandomSearch(w.expr, w.pars, w.consts, w.M, torch.float32)
    rs.setup(_t(prot), _t(data), _t(lb), _t(ub))
    rs.run(300, seed=1234)
    torch.cuda.synchronize()
    om = OracleModel(w.expr, w.pars, w.consts)
    bp = np.ascontiguousarray(np.broadcast_to(lb[:, None], (4, 4096)))
    bf = np.full(4096, np.finfo(np.float32).max / 5, np.float32)
    om.random_search(prot, data, lb, ub, bp, bf, 300, 0, seed=1234)
    got_f = rs.best_f_t.cpu().numpy()[0]
    # identical draws; costs differ only by expf rounding, so the same draw wins
    same = np.isclose(got_f, bf, rtol=1e-5)
    assert same.mean() > 0.995
    assert np.mean(np.all(np.isclose(rs.best_pars_t.cpu().numpy(), bp, rtol=1e-6), axis=0)) > 0.995
    # a second run continues from the best so far and never gets worse
    before = rs.best_f_t.clone()
    rs.run(50)
    torch.cuda.synchronize()
    assert bool((rs.best_f_t <= before).all())


def test_second_order_random_search_vs_oracle(ivim_data):
    w, data, lb, ub, prot = ivim_data
    rs = SecondOrderRandomSearch(w.expr, w.pars, w.consts, w.M, torch.float32)
    rs.setup(_t(prot), _t(data), _t(lb), _t(ub))
    rs.run(8, lm_iters=15, seed=99)
    torch.cuda.synchronize()
    om = OracleModel(w.expr, w.pars, w.consts)
    bp = np.ascontiguousarray(np.broadcast_to(lb[:, None], (4, 4096)))
    bf = np.full(4096, np.finfo(np.float32).max / 5, np.float32)
    om.random_search(prot, data, lb, ub, bp, bf, 8, 15, seed=99, solve_dtype=np.float64)
    got = rs.best_f_t.cpu().numpy()[0]
    rel = parity.rel_err(got, bf)
    assert np.median(rel) < 1e-5 and np.mean(rel < 1e-3) > 0.9, (np.median(rel), np.mean(rel < 1e-3))
    # refining the same 8 draws with the LM lowers the cost by orders of magnitude
    plain = RandomSearch(w.expr, w.pars, w.consts, w.M, torch.float32)
    plain.setup(_t(prot), _t(data), _t(lb), _t(ub))
    plain.run(8, seed=99)
    torch.cuda.synchronize()
    assert np.median(got) < 0.05 * np.median(plain.best_f_t.cpu().numpy())
