"""The C-ABI library loads here (no GPU) and exports what include/*.h declares;
the options struct is byte-identical to the reference's; host-side logic that
needs no device (defaults, argument checks) behaves as the reference's."""
import ctypes
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_functions():
    names = []
    for h in ("cufinufft.h",):
        txt = open(os.path.join(ROOT, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"\bint\s+(cufinufftf?_\w+)\s*\(", txt)
    return sorted(set(names))


@pytest.fixture(scope="module")
def lib():
    from cufinufft_gb300 import _cufinufft
    return _cufinufft.lib


def test_library_exports_every_declared_symbol(lib):
    names = _declared_functions()
    # the ten reference entry points (include/cufinufft_eitherprec.h:311-324)
    for base in ("default_opts", "makeplan", "setpts", "execute", "destroy"):
        assert f"cufinufft_{base}" in names and f"cufinufftf_{base}" in names
    for n in names:
        assert hasattr(lib, n), n


def test_opts_layout_matches_reference():
    from cufinufft_gb300._cufinufft import NufftOpts
    # include/cufinufft_opts.h:4-26: one double then 13 ints
    fields = [f for f, _ in NufftOpts._fields_]
    assert fields == ["upsampfac", "gpu_method", "gpu_sort", "gpu_binsizex", "gpu_binsizey",
                      "gpu_binsizez", "gpu_obinsizex", "gpu_obinsizey", "gpu_obinsizez",
                      "gpu_maxsubprobsize", "gpu_nstreams", "gpu_kerevalmeth",
                      "gpu_spreadinterponly", "gpu_device_id"]
    assert ctypes.sizeof(NufftOpts) == 64
    assert NufftOpts.gpu_method.offset == 8
    assert NufftOpts.gpu_device_id.offset == 8 + 12 * 4


@pytest.mark.parametrize("dim", [1, 2, 3])
@pytest.mark.parametrize("ntype", [1, 2])
def test_default_opts_match_reference(lib, dim, ntype):
    from cufinufft_gb300._cufinufft import NufftOpts, _default_opts, _default_optsf
    for fn in (_default_opts, _default_optsf):
        o = NufftOpts()
        assert fn(ntype, dim, o) == 0
        # src/cufinufft.cu:639-730
        assert o.upsampfac == 2.0
        assert o.gpu_method == (2 if ntype == 1 else 1)
        assert o.gpu_sort == 1
        assert o.gpu_maxsubprobsize == 1024
        assert (o.gpu_binsizex, o.gpu_binsizey, o.gpu_binsizez) == (-1, -1, -1)
        assert (o.gpu_obinsizex, o.gpu_obinsizey, o.gpu_obinsizez) == (-1, -1, -1)
        assert o.gpu_kerevalmeth == 0 and o.gpu_spreadinterponly == 0
        assert o.gpu_nstreams == 0 and o.gpu_device_id == 0


def test_default_opts_type3(lib):
    # the reference reserves type 3 and returns 1 here (src/cufinufft.cu:
    # 685-689); type 3 is implemented in this library and spreads as type 1
    from cufinufft_gb300._cufinufft import NufftOpts, _default_opts
    o = NufftOpts()
    assert _default_opts(3, 2, o) == 0
    assert o.gpu_method == 2 and o.upsampfac == 2.0
    assert _default_opts(4, 2, NufftOpts()) == 1


def test_makeplan_argument_checks_need_no_device(lib):
    from cufinufft_gb300._cufinufft import _make_planf
    plan = ctypes.c_void_p(None)
    nmodes = (ctypes.c_int * 3)(16, 16, 1)
    # bad dim / bad ntransf / bad modes are rejected before any CUDA call
    assert _make_planf(1, 4, nmodes, 1, 1, 1e-6, 0, ctypes.byref(plan), None) != 0
    assert plan.value is None
    assert _make_planf(1, 2, nmodes, 1, 0, 1e-6, 0, ctypes.byref(plan), None) != 0
    bad = (ctypes.c_int * 3)(0, 16, 1)
    assert _make_planf(1, 2, bad, 1, 1, 1e-6, 0, ctypes.byref(plan), None) != 0


def test_null_plan_calls_fail_cleanly(lib):
    from cufinufft_gb300._cufinufft import _destroy_plan, _destroy_planf, _exec_planf, _set_ptsf
    assert _destroy_plan(None) == 1   # reference: cannot destroy a NULL plan
    assert _destroy_planf(None) == 1
    assert _set_ptsf(10, None, None, None, 0, None, None, None, None) != 0
    assert _exec_planf(None, None, None) != 0


def test_python_wrapper_rejects_unknown_option(lib):
    # python/cufinufft/tests/test_error_checks.py:66-69: raised before any
    # device work
    from cufinufft_gb300 import cufinufft
    with pytest.raises(TypeError) as err:
        cufinufft(1, (8, 8), foo="bar")
    assert "Invalid option 'foo'" in err.value.args[0]
    with pytest.raises(TypeError):
        cufinufft(1, (8, 8), dtype=np.int32)


def _struct_fields(header, name):
    """Field names and C types of `typedef struct name { ... } name;` in order."""
    txt = open(os.path.join(ROOT, "include", header)).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    body = re.search(r"typedef struct " + name + r"\s*\{(.*?)\}\s*" + name + ";", txt, flags=re.S).group(1)
    fields = []
    for decl in body.split(";"):
        decl = decl.strip()
        if not decl:
            continue
        ctype, names = decl.split(None, 1)
        fields += [(n.strip(), ctype) for n in names.split(",")]
    return fields


def test_plan_info_mirror_matches_header():
    """The Python mirror of cufinufft_plan_info (an extension struct) has the
    header's fields in the header's order, with the same C types."""
    from cufinufft_gb300._cufinufft import PlanInfo
    want = _struct_fields("cufinufft.h", "cufinufft_plan_info")
    ct = {"int": ctypes.c_int, "double": ctypes.c_double}
    got = [(f, t) for f, t in PlanInfo._fields_]
    assert [f for f, _ in got] == [f for f, _ in want]
    for (f, t), (_, c) in zip(got, want):
        assert t == ct[c], f


@pytest.mark.parametrize("header,name,mirror", [
    ("cufinufft.h", "cufinufft_tune_entry", "TuneEntry"),
    ("cufinufft_opts.h", "cufinufft_opts", "NufftOpts"),
])
def test_other_struct_mirrors_match_headers(header, name, mirror):
    from cufinufft_gb300 import _cufinufft
    want = _struct_fields(header, name)
    ct = {"int": ctypes.c_int, "double": ctypes.c_double, "float": ctypes.c_float}
    got = getattr(_cufinufft, mirror)._fields_
    assert [f for f, _ in got] == [f for f, _ in want]
    for (f, t), (_, c) in zip(got, want):
        assert t == ct[c], f
