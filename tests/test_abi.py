"""CPU tests of the C ABI library: it loads, exports every symbol include/sfgpu.h declares, and its host-only
entry points (options, collider) behave; no GPU compute is called."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT, pkg, scenes

HEADER = os.path.join(ROOT, "include", "sfgpu.h")


def declared_symbols():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"SF_EXPORT\s+[\w\s\*]*?\b(sf_\w+)\s*\(", txt)))


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["sf_create", "sf_destroy", "sf_pressure_project", "sf_pressure_project_dev", "sf_pressure_reproject",
              "sf_magnetic_solve", "sf_magnetic_solve_dev", "sf_collider_box_fractions"]:
        assert s in syms


def test_library_exports_every_declared_symbol():
    lib = pkg().load_library()
    so = pkg()._abi.LIB_PATH
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT\s+(sf_\w+)", out))
    for s in declared_symbols():
        assert s in exported, s
        assert hasattr(lib, s)
    assert set(pkg()._abi.EXPORTED) == set(declared_symbols())


def test_abi_version_and_defaults():
    sf = pkg()
    lib = sf.load_library()
    assert lib.sf_abi_version() == 2
    o = sf.options("pressure")
    assert o.tol == 1e-8 and o.precision == sf.SF_PREC_FP64 and o.warm_start == 1
    m = sf.options("magnetic", precision="mixed")
    assert m.tol == 1e-6 and m.precision == sf.SF_PREC_MIXED
    assert lib.sf_status_string(0) == b"ok"
    assert lib.sf_status_string(1) == b"not converged"
    # mixed-form defaults: colour-split finest level, 48 coarsest pairs, the fused coarse tail, coarse sweeps as
    # pre / post
    assert (m.smoother, m.coarse_sweeps, m.coarse_tail, m.coarse_pre, m.coarse_post) == (3, 48, 0, 0, 0)
    assert m.inner_tol == 1e-3 and m.coarse_dim == 8 and m.pre_smooth == 2 and m.post_smooth == 2


def test_solve_opts_field_offsets_match_header():
    """Every field of the ctypes sf_solve_opts sits at the C offset (compiled offsetof probe)."""
    sf = pkg()
    O = sf._abi.sf_solve_opts
    names = [f for f, _ in O._fields_]
    body = "".join(f'printf("%zu\\n", offsetof(sf_solve_opts, {f}));' for f in names)
    src = '#include "sfgpu.h"\n#include <stdio.h>\n#include <stddef.h>\nint main(){' + body + 'return 0;}\n'
    tmp = os.path.join(ROOT, "oracle", "_build")
    os.makedirs(tmp, exist_ok=True)
    c = os.path.join(tmp, "offsets.c")
    exe = os.path.join(tmp, "offsets")
    open(c, "w").write(src)
    subprocess.check_call(["gcc", "-I" + os.path.join(ROOT, "include"), c, "-o", exe])
    offs = [int(v) for v in subprocess.check_output([exe]).split()]
    assert offs == [getattr(O, f).offset for f in names]


def test_structs_match_header_sizes():
    """ctypes mirrors of sf_grid / sf_solve_opts / sf_solve_stats have the C sizes (compiled probe)."""
    sf = pkg()
    src = '#include "sfgpu.h"\n#include <stdio.h>\nint main(){printf("%zu %zu %zu\\n", sizeof(sf_grid), ' \
          'sizeof(sf_solve_opts), sizeof(sf_solve_stats));return 0;}\n'
    tmp = os.path.join(ROOT, "oracle", "_build")
    os.makedirs(tmp, exist_ok=True)
    c = os.path.join(tmp, "sizes.c")
    exe = os.path.join(tmp, "sizes")
    open(c, "w").write(src)
    subprocess.check_call(["gcc", "-I" + os.path.join(ROOT, "include"), c, "-o", exe])
    sizes = [int(v) for v in subprocess.check_output([exe]).split()]
    assert sizes == [C.sizeof(sf._abi.sf_grid), C.sizeof(sf._abi.sf_solve_opts), C.sizeof(sf._abi.sf_solve_stats)]


def test_create_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = pkg().load_library()
    h = C.c_void_p()
    assert lib.sf_create(0, None, C.byref(h)) == 4  # SF_NO_DEVICE
    assert not h.value


def test_bad_arguments_rejected_without_gpu():
    lib = pkg().load_library()
    nulls = pkg()._abi.p3([0, 0, 0])
    assert lib.sf_collider_box_fractions(None, 0, nulls, None) == 2  # SF_BAD_ARG
    g = pkg().StaggeredGrid.from_origin(0.1, (4, 4, 4)).c_grid()
    assert lib.sf_collider_box_fractions(C.byref(g), -1, nulls, None) == 2
    assert lib.sf_collider_box_fractions(C.byref(g), 0, nulls, None) == 2


def test_noalloc_rejects_bad_arguments_before_any_device_call():
    """sf_magnetic_residual_noalloc checks its arguments on the host first: a null hext entry, band_width <= 0 or
    not finite, a non-finite chi and a null output are SF_BAD_ARG without touching a device (the pointers are
    never dereferenced on these paths)."""
    lib = pkg().load_library()
    abi = pkg()._abi
    g = pkg().StaggeredGrid.from_origin(0.1, (8, 8, 8)).c_grid()
    fake = 4096  # any non-null address: rejected before use
    ok3 = abi.p3([fake, fake, fake])

    def call(hext=ok3, chi=1.0, bw=0.2, phi=fake, psi=fake, result=fake):
        return lib.sf_magnetic_residual_noalloc(None, C.byref(g), C.c_void_p(phi), chi, bw, hext,
                                                C.c_void_p(psi), C.c_void_p(result))

    for a in range(3):
        h = [fake, fake, fake]
        h[a] = 0
        assert call(hext=abi.p3(h)) == abi.SF_BAD_ARG
    for bw in (0.0, -0.1, float("nan"), float("inf")):
        assert call(bw=bw) == abi.SF_BAD_ARG
    assert call(chi=float("nan")) == abi.SF_BAD_ARG
    assert call(phi=0) == abi.SF_BAD_ARG and call(psi=0) == abi.SF_BAD_ARG and call(result=0) == abi.SF_BAD_ARG


def test_every_declared_symbol_has_a_binding():
    """The ctypes binding gives every entry point of the header its argument types (a wrong or missing one
    passes arguments as C ints), and its list of exported names is the header's."""
    lib = pkg().load_library()
    syms = declared_symbols()
    for s in syms:
        assert getattr(lib, s).argtypes is not None, s
    assert sorted(pkg()._abi.EXPORTED) == syms


def test_prefetch_rejects_bad_arguments_before_any_device_call():
    """sf_applied_field_prefetch checks its arguments on the host: a null context, grid or field pointer, or a
    null field entry, is SF_BAD_ARG without touching a device."""
    lib = pkg().load_library()
    abi = pkg()._abi
    g = pkg().StaggeredGrid.from_origin(0.1, (8, 8, 8)).c_grid()
    fake = 4096
    assert lib.sf_applied_field_prefetch(None, C.byref(g), abi.p3([fake, fake, fake])) == abi.SF_BAD_ARG


def test_package_has_no_cpu_fallback(monkeypatch):
    """The package raises when the library is missing instead of computing on the CPU."""
    sf = pkg()
    monkeypatch.setattr(sf._abi, "_lib", None)
    with pytest.raises(ImportError):
        sf._abi.load("/nonexistent/libsfgpu.so")
