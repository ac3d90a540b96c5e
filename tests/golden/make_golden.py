"""Generate the golden fixtures of the IVIM fitter from the reference's own kernel.

Runs the reference's generated LM kernel
``test/ivim/second_order_levenberg_marquardt_4_1_21_f_f7def86f0a03.cu`` (built
as host C++ into oracle/_ref by oracle/Makefile; the 10- and 16-sample builds
rewrite only its sample count) on seeded synthetic IVIM inputs and stores inputs and
outputs as small .npz files:

  ivim{21,10,16}_it1.npz    one iteration (every quantity deterministic to ~1 ulp)
  ivim{21,10,16}_it100.npz  100 iterations (the benchmark iteration count)
  ivim21_search.npz      one SearchStep launch of the random-search kernel

Needs the reference tree (PCGB_REFERENCE_TREE, or a `reference` directory
beside this repository):
    python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import RefIVIM, build_reference  # noqa: E402
from pycompute_gb300 import synth  # noqa: E402

N = 512
SEED = 20240611


def main():
    from __graft_entry__ import reference_tree

    ref_root = reference_tree()
    if not ref_root or not build_reference(ref_root):
        raise SystemExit("reference tree not found (set PCGB_REFERENCE_TREE); fixtures are generated where it exists")
    for M, bvals in ((21, synth.IVIM_B21), (10, synth.IVIM_B10), (16, synth.ivim_b16())):
        w = synth.ivim(bvals, name=f"ivim{M}")
        true, data, init, lb, ub, prot = w.generate(N, seed=SEED + M)
        ref = RefIVIM(M)
        for iters in (1, 100):
            p = init.copy()
            out = ref.lm_run(p, prot, data, lb, ub, iters, want_step=True)
            np.savez_compressed(
                os.path.join(HERE, f"ivim{M}_it{iters}.npz"),
                expr=w.expr, pars_str=np.array(w.pars), consts_str=np.array(w.consts),
                protocol=prot, data=data, init=init, lb=lb, ub=ub, true=true, iters=iters,
                tol=1e-8, mu=0.25, eta=0.75, acc=0.2, dec=2.0,
                pars=out["pars"], lam=out["lam"], step_type=out["step_type"], f=out["f"],
                first_f=out["first_f"], last_f=out["last_f"], step=out["step"])
            print(f"ivim{M}_it{iters}: converged {np.mean(out['step_type'] == 0):.4f}")
    # one SearchStep launch: cost at random points, keep the best
    w = synth.ivim(synth.IVIM_B21)
    true, data, init, lb, ub, prot = w.generate(N, seed=SEED + 7)
    rng = np.random.default_rng(SEED)
    lbv = np.broadcast_to(lb[:, None], (4, N)).astype(np.float32)
    ubv = np.broadcast_to(ub[:, None], (4, N)).astype(np.float32)
    p = (lbv + rng.random((4, N), dtype=np.float32) * (ubv - lbv)).astype(np.float32)
    best_p = init.copy()
    best_f = np.full(N, np.finfo(np.float32).max / 5, dtype=np.float32)
    best_f[: N // 2] = 1e5
    f = np.zeros(N, dtype=np.float32)
    consts = np.ascontiguousarray(np.broadcast_to(prot[:, None], (21, N)))
    p_in, best_p_in, best_f_in = p.copy(), best_p.copy(), best_f.copy()
    RefIVIM(21).search_step(consts, data, np.ascontiguousarray(lbv), np.ascontiguousarray(ubv), best_p, p, best_f, f)
    np.savez_compressed(os.path.join(HERE, "ivim21_search.npz"), protocol=prot, data=data, p=p_in, best_p_in=best_p_in,
                        best_f_in=best_f_in, best_p=best_p, best_f=best_f, f=f)
    print("ivim21_search written")


if __name__ == "__main__":
    main()
