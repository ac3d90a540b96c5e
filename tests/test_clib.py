"""libpcgb.so: loads without a GPU, exports every entry point of include/pcgb.h,
compiles fitter programs with NVRTC for sm_103a, and rejects bad arguments
with an error code and message instead of crashing."""
import ctypes
import os
import re

import pytest

from pycompute_gb300 import _lib, codegen, synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for fn in sorted(os.listdir(os.path.join(ROOT, "include"))):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names += re.findall(r"\b(pcgb_[a-z0-9_]+)\s*\(", text)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = _lib.lib()
    declared = _declared()
    assert len(declared) >= 10
    for name in declared:
        assert hasattr(L, name), name
    assert set(declared) == set(_lib.SIGNATURES), "ctypes signatures out of sync with the header"


def test_version_and_limits():
    L = _lib.lib()
    assert b"sm_103a" in L.pcgb_version()
    assert L.pcgb_max_params() == 8
    assert L.pcgb_max_protocol() >= 64


def _compile(gm, M, dt=0, sdt=1):
    L = _lib.lib()
    buf = ctypes.create_string_buffer(1 << 16)
    rc = L.pcgb_fitter_compile(gm.source.encode(), gm.struct_name.encode(), gm.P, gm.C, M, dt, sdt,
                               _lib.cache_dir().encode(), buf, len(buf))
    return rc, buf.value.decode(), L.pcgb_last_error().decode()


def test_nvrtc_compiles_ivim_for_sm103a_within_spill_cap():
    """The LM kernels for a shared protocol are built for 6 resident blocks
    per SM (the warm LM with its check epilogue for 7); their spills stay
    under the 256-byte cap for the fp32-state builds, and a build over the cap
    (the all-FP64 one) is followed by the uncapped build, which does not
    spill. Groups served from the cubin cache print no log."""
    import re
    w = synth.ivim()
    gm = codegen.generate(w.expr, w.pars, w.consts)
    for dt, sdt in ((0, 1), (0, 0), (1, 1)):
        rc, log, err = _compile(gm, w.M, dt, sdt)
        assert rc == 0, err
        for kernel in ("pcgb_lm_c1_b1", "pcgb_lmw_c1_b1"):
            blocks = log.split(f"Function properties for {kernel}\n")[1:]
            if not blocks:  # that group came from the cubin cache
                continue
            spills = [int(re.search(r"(\d+) bytes spill stores", b).group(1)) for b in blocks]
            if dt == 0:
                assert spills[0] <= 256, (kernel, spills)
            if spills[0] > 256:
                assert len(spills) >= 2 and spills[1] == 0, (kernel, spills)


def test_ivim16_fit_and_refit_kernels_keep_the_register_cap(tmp_path):
    """IVIM-16, fp32 state and FP64 solve (the warm-start workload): the fit
    kernel and the fallback refit + select kernel are both kept at the
    6-blocks-per-SM register cap (80 registers). The refit shares no program
    with the check-epilogue and refill kernels, which spill past the cap and
    have their own group rebuilt without it."""
    w = synth.ivim(synth.ivim_b16(), name="ivim16")
    gm = codegen.generate(w.expr, w.pars, w.consts)
    L = _lib.lib()
    buf = ctypes.create_string_buffer(1 << 21)
    rc = L.pcgb_fitter_compile(gm.source.encode(), gm.struct_name.encode(), gm.P, gm.C, w.M, 0, 1,
                               str(tmp_path).encode(), buf, len(buf))
    assert rc == 0, L.pcgb_last_error().decode()
    log = buf.value.decode()

    def registers(kernel):  # of the build the runtime loads: the last one in the log
        block = log.split(f"Function properties for {kernel}\n")[-1]
        return int(re.search(r"Used (\d+) registers", block).group(1))

    assert registers("pcgb_lm_c1_b1") <= 80
    assert registers("pcgb_lms_c1_b1") <= 80


def test_compile_errors_are_reported():
    rc, _, err = _compile(codegen.GeneratedModel(expr="x", pars=["a"], consts=[], struct_name="Nope",
                                                 source="struct Nope { this is not C++ };", jnz=[True],
                                                 hnz=[False]), 4)
    assert rc == -1001 and "NVRTC" in err


@pytest.mark.parametrize("P,C,M,dt,sdt,code", [
    (0, 1, 10, 0, 1, -34), (9, 1, 10, 0, 1, -34), (4, 1, 0, 0, 1, -34), (4, 2, 200, 0, 1, -34),
    (4, 1, 10, 2, 1, -22), (4, 1, 10, 1, 0, -22)])
def test_create_argument_validation(P, C, M, dt, sdt, code):
    L = _lib.lib()
    h = ctypes.c_void_p()
    rc = L.pcgb_fitter_create(b"struct X{};", b"X", P, C, M, dt, sdt, None, ctypes.byref(h))
    assert rc == code and not h.value
    assert L.pcgb_last_error()


def test_run_rejects_null_fitter():
    L = _lib.lib()
    rc = L.pcgb_lm_run(None, None, 0, None, None, None, 0, 1e-8, .25, .75, .2, 2., None, None, None, None, None,
                       None, None, None, 10, 10, None, 0, None, None, 0, None)
    assert rc == -22 and b"NULL" in L.pcgb_last_error()
    assert L.pcgb_fitter_destroy(None) == 0


def test_elementwise_gelu_rejects_bad_arguments_without_a_gpu():
    L = _lib.lib()
    assert L.pcgb_mlp_gelu(None, 0, 0, None, None, None) == 0
    assert L.pcgb_mlp_gelu(None, 5, 0, None, None, None) == -22
    assert L.pcgb_mlp_last_error()
    assert L.pcgb_mlp_gelu(None, -1, 0, None, None, None) == -22
    assert L.pcgb_mlp_gelu(None, 0, -1, None, None, None) == -22


@pytest.mark.parametrize("entry", ["pcgb_multi_run", "pcgb_multi_run_noalloc"])
def test_mixed_run_refuses_more_than_2_31_chunks_before_any_gpu_work(entry):
    """Both mixed-model entry points refuse a request whose chunk count would
    let the 32-bit work counter wrap (2^31 chunks over all jobs, summed without
    overflow), before they look at the program or touch the GPU: here no
    program and no GPU exist at all."""
    from pycompute_gb300.multi import _Job

    L = _lib.lib()
    cases = [[(1 << 31) * 64 + 1], [1 << 62, 1 << 62], [(1 << 63) - 1, (1 << 63) - 1], [(1 << 30) * 64] * 3]
    for sizes in cases:
        arr = (_Job * len(sizes))()
        for j, n in zip(arr, sizes):
            j.nprobs = n
        args = [None, arr, len(sizes), None, 1, 1e-8, 0.25, 0.75, 0.2, 2.0, 64, 0]
        rc = getattr(L, entry)(*args, *([None] if entry == "pcgb_multi_run" else []), None)
        assert rc == -34, (sizes, rc)
        err = L.pcgb_noalloc_last_error() if entry.endswith("noalloc") else L.pcgb_last_error()
        assert b"2^31" in err
    # exactly 2^31 chunks passes the range check and fails on the missing program
    arr = (_Job * 1)()
    arr[0].nprobs = (1 << 31) * 64
    rc = getattr(L, entry)(None, arr, 1, None, 1, 1e-8, 0.25, 0.75, 0.2, 2.0, 64, 0,
                           *([None] if entry == "pcgb_multi_run" else []), None)
    assert rc != -34


@pytest.mark.parametrize("entry", ["pcgb_gemm_bf16_tc", "pcgb_gemm_bf16"])
def test_training_gemms_refuse_misaligned_operands_before_any_gpu_work(entry):
    """Both training-GEMM entry points read their operands in 16-byte chunks:
    a pointer off a 16-byte boundary is refused with EINVAL before anything
    is read or launched (the pointers here point at nothing)."""
    L = _lib.lib()
    fake = ctypes.c_void_p
    err = L.pcgb_gemm_tc_last_error if entry.endswith("_tc") else L.pcgb_mlp_last_error
    for a, b in ((0x10008, 0x20000), (0x10000, 0x20002)):
        args = [0, 0, 1, fake(a), 16, fake(b), 16, 64, 8, 16, 0, fake(0x30000), 17, fake(0x40000), 8, None, 0,
                None, 0]
        rc = getattr(L, entry)(*args, *([None] if entry.endswith("_tc") else []), None)
        assert rc == -22, (a, b, rc)
        assert b"16-byte aligned" in err()
