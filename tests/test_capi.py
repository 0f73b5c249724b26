"""The C-ABI library: loads without a GPU, exports every declared symbol, host-only entry points (no GPU)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import oracle as O
from conftest import ROOT


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        names |= set(re.findall(r"\b(pmg_\w+)\s*\(", text))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    from pymoto_gb300 import _lib
    return _lib.load()


def test_every_declared_symbol_is_exported(lib):
    names = declared_symbols()
    assert len(names) > 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_the_header():
    from pymoto_gb300 import _lib
    assert set(declared_symbols()) == set(_lib.SIGNATURES)


def test_version_and_status_strings(lib):
    from pymoto_gb300 import _lib
    assert _lib.call("pmg_version") >= 100
    assert lib.pmg_status_string(1) == b"invalid argument"
    assert lib.pmg_status_string(5) == b"matrix not positive definite"


@pytest.mark.parametrize("dim,plane,units", [(2, "strain", (1, 1, 1)), (2, "stress", (0.5, 2.0, 0.3)),
                                             (3, "strain", (1, 1, 1)), (3, "strain", (0.1, 0.2, 0.3))])
def test_element_stiffness_matches_oracle(dim, plane, units):
    from pymoto_gb300 import element_stiffness
    g = O.Grid(2, 2, 2 if dim == 3 else 0, *units)
    ref = O.element_stiffness(g, plane=plane)
    np.testing.assert_allclose(element_stiffness(dim, plane=plane, unit=units), ref, rtol=0,
                               atol=1e-15 * np.abs(ref).max())


@pytest.mark.parametrize("dim", [2, 3])
def test_galerkin_table_is_child_transfer_product(dim):
    """table[s] = M_s^T K0 M_s with M_s the restriction of R to child s of one coarse cell."""
    from pymoto_gb300._lib import call
    g = O.Grid(2, 2, 2 if dim == 3 else 0)
    K0 = O.element_stiffness(g)
    nde = K0.shape[0]
    table = np.zeros((2 ** dim, nde, nde))
    call("pmg_galerkin_table", dim, K0, table)
    R = O.prolongation(g).toarray()          # fine 2x2(x2) grid -> coarse 1x1(x1) grid
    fine_dc = g.dofconn()
    cg = g.coarse()
    coarse_dc = cg.dofconn()[0]
    for s in range(2 ** dim):
        M = R[np.ix_(fine_dc[g.elem_number(s & 1, (s >> 1) & 1, (s >> 2) & 1 if dim == 3 else 0)], coarse_dc)]
        np.testing.assert_allclose(table[s], M.T @ K0 @ M, rtol=0, atol=1e-14 * np.abs(K0).max())


@pytest.mark.parametrize("shape", [(8, 4, 4), (4, 8, 2), (6, 0, 0), (3, 5, 0), (2, 2, 6)])
def test_coarse_ordering_is_a_band_reducing_permutation(shape):
    """pmg_coarse_ordering: a permutation of the dofs under which every stencil coupling of the grid (the
    nonzeros of the coarsest matrix) lies within the reported half bandwidth, at most the natural one."""
    from pymoto_gb300._lib import call
    nx, ny, nz = shape
    if ny == 0:
        ny = nx
    g = O.Grid(nx, ny, nz)
    n = g.nnodes * g.dim
    pos = np.empty(n, dtype=np.int32)
    bw = np.zeros(1, dtype=np.int32)
    call("pmg_coarse_ordering", nx, ny, nz, pos, bw)
    assert np.array_equal(np.sort(pos), np.arange(n))
    K = O.assemble(g, O.element_stiffness(g), np.ones(g.nel), np.zeros(0, dtype=np.int64)).tocoo()
    band = np.abs(pos[K.row] - pos[K.col]).max()
    assert band <= bw[0] <= call("pmg_stencil_bandwidth", nx, ny, nz)
    if shape == (8, 4, 4):                    # the coarsest grid of a 128 x 64 x 64 five-level hierarchy
        assert (call("pmg_stencil_bandwidth", nx, ny, nz), int(bw[0])) == (167, 95)


def test_invalid_arguments_fail_before_any_launch():
    from pymoto_gb300._lib import PMGError, call
    with pytest.raises(PMGError) as e:
        call("pmg_ebe_apply", 0, 0, 0, 4, 4, None, None, None, 1.0, None, None, None, 0.0, None, None, None)
    assert e.value.status == 1
    with pytest.raises(PMGError):
        call("pmg_restrict", 0, 5, 4, 0, None, None, None)      # odd grid
    with pytest.raises(PMGError):
        call("pmg_conv_filter", 4, 4, 0, None, 2, 1, 1, None, None, None, None, None, None)
    with pytest.raises(PMGError):
        call("pmg_element_stiffness", 4, 1.0, 0.3, 0, 1.0, 1.0, 1.0, np.zeros(4))
    assert call("pmg_stencil_bandwidth", 2, 1, 1) == (1 + 3 + 3 * 2) * 3 + 2


def test_noalloc_dot_rejects_bad_arguments_without_a_gpu():
    """pmg_dot_noalloc checks its arguments before it touches the device: null pointers, an unknown dtype,
    a negative or too large n are PMG_BAD_ARG."""
    from pymoto_gb300._lib import PMGError, call
    buf = np.zeros(4)
    bad = [(0, 4, None, buf, buf), (0, 4, buf, None, buf), (0, 4, buf, buf, None), (7, 4, buf, buf, buf),
           (0, -1, buf, buf, buf), (0, 4_194_305, buf, buf, buf)]
    for dtype, n, a, b, out in bad:
        with pytest.raises(PMGError) as e:
            call("pmg_dot_noalloc", dtype, n, a, b, out, None)
        assert e.value.status == 1, (dtype, n)


def test_product_package_never_imports_the_oracle():
    pkg = os.path.join(ROOT, "pymoto_gb300")
    for path in glob.glob(os.path.join(pkg, "**", "*.py"), recursive=True):
        src = open(path).read()
        assert not re.search(r"^\s*(import|from)\s+oracle\b", src, flags=re.M), path


def _header_prototypes():
    """name -> (return type, [parameter types]) of every function declared in include/*.h."""
    protos = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        text = re.sub(r"//[^\n]*", "", text)
        for m in re.finditer(r"([A-Za-z_][\w\s\*]*?)\b(pmg_\w+)\s*\(([^;{]*?)\)\s*;", text):
            ret, name, params = m.group(1).strip(), m.group(2), m.group(3).strip()
            plist = [] if params in ("", "void") else [p.strip() for p in params.split(",")]
            types = []
            for p in plist:
                p = re.sub(r"\s+", " ", p)
                if "*" in p:
                    types.append("ptr")
                else:
                    types.append(p.rsplit(" ", 1)[0].replace("const ", "").strip())
            protos[name] = (ret.split()[-1] if "*" not in ret else "ptr", types)
    return protos


def test_binding_signatures_match_the_header():
    """Argument count and type class of every ctypes signature against its C declaration: a mismatch would pass
    wrong values (or pointers) to the library."""
    from pymoto_gb300 import _lib
    cmap = {"int": ctypes.c_int, "int64_t": ctypes.c_int64, "double": ctypes.c_double, "float": ctypes.c_float,
            "size_t": ctypes.c_size_t, "unsigned": ctypes.c_uint}
    protos = _header_prototypes()
    assert set(protos) == set(_lib.SIGNATURES)
    bad = []
    for name, (res, args) in _lib.SIGNATURES.items():
        ret, types = protos[name]
        if len(types) != len(args):
            bad.append(f"{name}: {len(types)} declared, {len(args)} bound")
            continue
        for k, (t, a) in enumerate(zip(types, args)):
            if t == "ptr":
                ok = a in (ctypes.c_void_p, ctypes.c_char_p)
            else:
                ok = cmap.get(t) is a
            if not ok:
                bad.append(f"{name} arg {k}: {t} vs {a.__name__}")
        want = ctypes.c_char_p if ret == "ptr" else cmap.get(ret)
        if want is not res:
            bad.append(f"{name} returns {ret} vs {getattr(res, '__name__', res)}")
    assert not bad, bad


def test_mma_and_overhang_arguments_are_checked_before_any_launch():
    """pmg_mma_update and pmg_overhang_* reject bad options before any launch (host buffers stand in for the
    device arrays: every case below returns at the option checks)."""
    import ctypes as C
    from pymoto_gb300._lib import PMGError, call
    from pymoto_gb300.mma import _Params
    n, m = 8, 1
    assert call("pmg_mma_scratch_bytes", 0, 1) == 0 and call("pmg_mma_scratch_bytes", n, 5) == 0
    s1, s2 = call("pmg_mma_scratch_bytes", n, 1), call("pmg_mma_scratch_bytes", 2 * n, 1)
    assert s2 - s1 == (12 + 2 * (m + 1) + m) * n * 8
    assert call("pmg_mma_scratch_bytes", n, 2) - s1 == 3 * n * 8
    buf = [np.zeros(64) for _ in range(14)]
    x, x1, x2, lo, hi, mv, g, dg, off, low, upp, xn, info, scr = buf

    def good():
        p = _Params()
        p.version, p.m, p.adapt, p.maxit, p.exact = 1, m, 0, 100, 0
        p.epsimin = 1e-7
        return p

    def update(p, **kw):
        args = dict(xval=x, xold1=x1, xold2=x2, xnew=xn)
        args.update(kw)
        return call("pmg_mma_update", n, C.byref(p), args["xval"], args["xold1"], args["xold2"], lo, hi, mv, g, dg,
                    off, low, upp, args["xnew"], info, scr, None)

    bad = []
    for field, value in (("m", 0), ("m", 5), ("maxit", 0), ("exact", 2), ("version", 3), ("epsimin", 0.0)):
        p = good()
        setattr(p, field, value)
        bad.append((p, {}))
    p = good()
    p.adapt = 1
    bad.append((p, {"xold1": None}))
    bad.append((good(), {"xnew": x}))                 # output aliases the design
    for p, kw in bad:
        with pytest.raises(PMGError) as e:
            update(p, **kw)
        assert e.value.status == 1
    # overhang: nx ny nz lay step layer w0 w1 w2 c0 c1 c2 K kern p q shift backshift eps x y s stream
    ok = [4, 4, 4, 1, 1, 0, 3, 1, 3, 1, 1, 1, 1]
    for i, v in ((3, 3), (4, 2), (5, 4), (6, 2), (7, 3), (8, 5), (10, -1), (12, 0)):
        a = list(ok)
        a[i] = v
        with pytest.raises(PMGError):
            call("pmg_overhang_forward", *a, buf[0], 40.0, 1.0, 0.5, 0.5, 1e-3, buf[1], buf[2], buf[3], None)
    with pytest.raises(PMGError):   # q must be positive
        call("pmg_overhang_forward", *ok, buf[0], 40.0, 0.0, 0.5, 0.5, 1e-3, buf[1], buf[2], buf[3], None)
    with pytest.raises(PMGError):   # output aliases the input
        call("pmg_overhang_forward", *ok, buf[0], 40.0, 1.0, 0.5, 0.5, 1e-3, buf[1], buf[1], buf[3], None)


def test_c_caller_without_python(tmp_path):
    """The header compiles as C99 and a C program linked against the library gets the element matrix and the
    argument checks from it (host-only calls: no GPU)."""
    import shutil
    import subprocess
    from pymoto_gb300 import _lib, element_stiffness
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    _lib.load()
    libdir = os.path.dirname(_lib.LIB_PATH)
    exe = str(tmp_path / "capi_host_check")
    subprocess.run([cc, "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "capi_host_check.c"), "-o", exe, "-L", libdir, "-lpymoto_gb300",
                    "-Wl,-rpath," + libdir], check=True, capture_output=True, text=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.splitlines()
    fields = dict(line.split(" ", 1) for line in out)
    assert int(fields["version"]) == _lib.call("pmg_version")
    assert fields["status"] == "invalid argument"
    K0 = np.array([float(v) for v in fields["K0"].split()]).reshape(24, 24)
    np.testing.assert_array_equal(K0, element_stiffness(3))
    assert int(fields["bad_mode"]) == 1 and int(fields["bad_grid"]) == 1


def test_operator_launch_plan_fits_the_kernel_limits():
    """The CUDA-core operator's launch plan (tile, tiles, z chunks) respects the kernel's thread, staging and grid
    limits and covers the node counts, for the bench grids and many others, without a GPU."""
    from pymoto_gb300 import _lib
    plan = np.zeros(5, dtype=np.int32)
    _lib.call("pmg_operator_plan", 128, 64, 64, 304, plan)
    assert plan.tolist() == [19, 13, 7, 5, 8]
    rng = np.random.default_rng(5)
    shapes = [(1, 1, 1), (2, 1, 1), (31, 1, 1), (32, 32, 32), (255, 3, 7), (256, 128, 128), (96, 48, 48),
              (4000, 2, 3), (3, 4000, 2)] + [tuple(int(v) for v in rng.integers(1, 300, 3)) for _ in range(300)]
    for nx, ny, nz in shapes:
        for slots in (1, 152, 304, 456):
            _lib.call("pmg_operator_plan", nx, ny, nz, slots, plan)
            ox, oy, tx, ty, nzc = plan.tolist()
            assert 1 <= ox <= 32 and 1 <= oy <= 32 and ox * oy <= 256, (nx, ny, nz, plan)
            assert (ox + 2) * (oy + 2) <= 340 and (ox + 1) * (oy + 1) <= 297, (nx, ny, nz, plan)
            assert tx * ox >= nx + 1 and (tx - 1) * ox < nx + 1, (nx, ny, nz, plan)
            assert ty * oy >= ny + 1 and (ty - 1) * oy < ny + 1, (nx, ny, nz, plan)
            assert 1 <= nzc <= min(nz + 1, 65535) and ty <= 65535, (nx, ny, nz, plan)
    with pytest.raises(_lib.PMGError):
        _lib.call("pmg_operator_plan", 8, 8, 0, 304, plan)


def test_every_called_entry_point_is_bound():
    """Every C-ABI name the package, the bench and the entry points call through the binding is declared and
    bound (a misspelt name would only fail on a GPU)."""
    from pymoto_gb300 import _lib
    files = glob.glob(os.path.join(ROOT, "pymoto_gb300", "*.py")) + [os.path.join(ROOT, "bench.py"),
                                                                      os.path.join(ROOT, "__graft_entry__.py")]
    called = set()
    for path in files:
        called |= set(re.findall(r"""call\(\s*["'](pmg_\w+)["']""", open(path).read()))
    assert len(called) > 50
    assert called <= set(_lib.SIGNATURES), sorted(called - set(_lib.SIGNATURES))
