"""CPU tests of the C ABI: libnsg.so builds, loads without a GPU, and exports
every function include/nsg.h declares."""
import os
import re
import subprocess

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared() -> set[str]:
    src = open(os.path.join(ROOT, "include", "nsg.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return set(re.findall(r"\b(nsg_[a-z0-9_]+)\s*\(", src))


def test_header_functions_are_exported(nsg):
    from nscale_gb300 import _lib
    names = declared()
    assert len(names) >= 25
    out = subprocess.run(["nm", "-D", "--defined-only", _lib.LIB_PATH], capture_output=True, text=True).stdout
    exported = set(re.findall(r" T (nsg_[a-z0-9_]+)", out))
    missing = names - exported
    assert not missing, f"declared but not exported: {sorted(missing)}"
    bound = set(_lib.exported_symbols())
    assert names <= bound, f"not bound in _lib: {sorted(names - bound)}"


def test_host_only_calls(nsg):
    import ctypes as C
    from nscale_gb300 import _lib
    assert nsg.nsg_version() >= 10000
    p = _lib.SegParams()
    nsg.nsg_default_params(C.byref(p))
    assert (p.blue, p.green, p.red, p.T1, p.T2, p.G1, p.minSize, p.maxSize, p.G2, p.minSizePl, p.minSizeSeg,
            p.maxSizeSeg, p.fillHolesConnectivity, p.reconConnectivity, p.watershedConnectivity) == \
        (220, 220, 220, 5.0, 4.0, 80, 11, 1000, 45, 30, 21, 1000, 4, 8, 8)
    assert nsg.nsg_status_string(3) == b"NO_CANDIDATES_LEFT"
    assert nsg.nsg_status_string(-12) == b"ERR_TIMEOUT"
    # argument errors are reported without touching a device
    assert nsg.nsg_context_create(None, 10, 10, 0) == _lib.ERR_ARG
    assert nsg.nsg_context_destroy(None) == _lib.ERR_ARG


def test_product_does_not_link_the_oracle(nsg):
    from nscale_gb300 import _lib
    out = subprocess.run(["nm", "-D", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "orc_" not in out and "ref_cc_" not in out
    deps = subprocess.run(["ldd", _lib.LIB_PATH], capture_output=True, text=True).stdout
    assert "oracle" not in deps and "torch" not in deps


def test_pool_and_server_host_checks(nsg):
    """Sizes and admission are decided on the host, before any device call."""
    import ctypes as C
    from nscale_gb300 import _lib
    per = nsg.nsg_pool_context_bytes(4096, 4096)
    assert per > 16 * 4096 * 4096  # several planes of the padded image
    assert nsg.nsg_pool_context_bytes(2048, 2048) < per
    assert nsg.nsg_pool_context_bytes(0, 10) == 0
    h = C.c_void_p()
    # a budget that does not hold one tile's workspace is refused
    assert nsg.nsg_server_create(C.byref(h), 4096, 4096, per - 1, 8, 0) == _lib.ERR_OOM
    assert nsg.nsg_server_create(C.byref(h), 4096, 4096, per, 0, 0) == _lib.ERR_ARG
    assert nsg.nsg_pool_create(C.byref(h), 512, 512, 0, 0) == _lib.ERR_ARG
    assert nsg.nsg_pool_destroy(None) == _lib.ERR_ARG
    assert nsg.nsg_server_destroy(None) == _lib.ERR_ARG
    assert nsg.nsg_segment_nuclei_batch(None, None, 0, None, 0) == _lib.ERR_ARG
    t = _lib.Tuning(0, 0, -1)
    assert nsg.nsg_context_set_tuning(None, C.byref(t)) == _lib.ERR_ARG
    assert nsg.nsg_pool_set_tuning(None, C.byref(t)) == _lib.ERR_ARG
    assert nsg.nsg_pool_set_timing(None, 1) == _lib.ERR_ARG
    assert nsg.nsg_pool_stage_times(None, None, 0, None) == _lib.ERR_ARG


def test_package_import_sets_hardware_queue_default():
    """Importing the package before CUDA starts asks for 32 hardware work
    queues (one per tile stream of the batched form); a caller's value wins."""
    import sys
    code = ("import os; os.environ.pop('CUDA_DEVICE_MAX_CONNECTIONS', None); import nscale_gb300; "
            "print(os.environ['CUDA_DEVICE_MAX_CONNECTIONS'])")
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT)
    assert out.stdout.strip() == "32", out.stderr
    env = dict(os.environ, CUDA_DEVICE_MAX_CONNECTIONS="4")
    code = "import os, nscale_gb300; print(os.environ['CUDA_DEVICE_MAX_CONNECTIONS'])"
    out = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, cwd=ROOT, env=env)
    assert out.stdout.strip() == "4", out.stderr


def test_autotune_worker_cap_follows_free_memory(nsg, monkeypatch):
    """max_workers: contexts that fit in the free device memory after a reserve
    (a quarter of it, at least 8 GiB), never fewer than one."""
    import torch
    from nscale_gb300 import _lib, autotune
    per = _lib.load().nsg_pool_context_bytes(4096, 4096)
    assert per > 0
    for free, want in [(280 << 30, int((280 * 0.75 * (1 << 30)) // per)), (16 << 30, int((8 << 30) // per)),
                       (1 << 30, 1)]:
        monkeypatch.setattr(torch.cuda, "mem_get_info", lambda device=0, f=free: (f, 288 << 30))
        assert autotune.max_workers(4096, 4096, 0) == max(1, want)
