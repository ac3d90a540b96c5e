"""The allocation-free mixed-model entry point, pcgb_multi_run_noalloc.

It is for callers that cannot allocate device memory (a host whose device
memory belongs to another framework's pool allocator, a service that reserves
its memory at start-up and may not grow it): it keeps the work counter in a
library-owned static device array instead of a caller-allocated word. Here it
is called through the C ABI twice in a row and must give the same fit as
pcgb_multi_run with a caller-provided counter, bit for bit on every voxel
(a voxel's fit does not depend on which warp claims its chunk). The file is
named so that pytest collects it last.
"""
import ctypes

import pytest
import torch

from pycompute_gb300 import Expr, _lib, synth
from pycompute_gb300.multi import MultiJob, MultiModelFitter, _Job

pytestmark = pytest.mark.gpu
DEV = "cuda:0"


def _setup():
    ws = [synth.t2star(), synth.ivim()]
    fitter = MultiModelFitter([(Expr(w.expr, w.pars, w.consts), w.M) for w in ws])
    jobs, inits = [], []
    for k, w in enumerate(ws):
        true, data, init, lb, ub, prot = w.generate(5000 + 37 * k, seed=40 + k)
        init_t = torch.from_numpy(init).to(DEV)
        jobs.append(MultiJob(init_t.clone(), torch.from_numpy(data).to(DEV), prot, lb, ub))
        inits.append(init_t)
    return fitter, jobs, inits


def _reset(jobs, inits):
    for j, i0 in zip(jobs, inits):
        j.reset(i0)


def _noalloc(fitter, jobs, iters, chunk=64):
    arr = (_Job * len(jobs))(*[j.ctype() for j in jobs])
    rc = _lib.lib().pcgb_multi_run_noalloc(fitter.build(), arr, len(jobs), None, iters, 1e-8, 0.25, 0.75, 0.2, 2.0,
                                           chunk, 0, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    _lib.check("pcgb_multi_run_noalloc", rc)


def test_noalloc_matches_caller_scratch_twice_in_a_row():
    fitter, jobs, inits = _setup()
    iters = 40
    fitter.fit(jobs, iters)  # caller-provided work counter
    torch.cuda.synchronize()
    want = [(j.pars.clone(), j.step_type.clone(), j.f.clone(), j.iters.clone()) for j in jobs]
    for _ in range(2):  # the shared counter must be cleared between calls
        _reset(jobs, inits)
        _noalloc(fitter, jobs, iters)
        torch.cuda.synchronize()
        for (p, st, f, it), j in zip(want, jobs):
            assert torch.equal(j.pars, p)
            assert torch.equal(j.step_type, st)
            assert torch.equal(j.f, f)
            assert torch.equal(j.iters, it)
            assert torch.all(j.iters > 0)


def test_noalloc_rejects_oversized_requests():
    fitter, jobs, inits = _setup()
    big = (_Job * 1)(jobs[0].ctype())
    big[0].nprobs = (1 << 31) * 64 + 1  # one chunk more than the counter's limit at chunk 64
    rc = _lib.lib().pcgb_multi_run_noalloc(fitter.build(), big, 1, None, 1, 1e-8, 0.25, 0.75, 0.2, 2.0, 64, 0,
                                           ctypes.c_void_p(torch.cuda.current_stream().cuda_stream))
    assert rc == -34
    assert b"2^31" in _lib.lib().pcgb_noalloc_last_error()
