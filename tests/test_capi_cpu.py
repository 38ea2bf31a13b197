"""The C-ABI library loads and exports every function include/*.h declares,
and the ctypes bindings match the header's signatures (no GPU needed)."""
import ctypes
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s*(fadesim_[a-z0-9_]+)\s*\(", src,
                             flags=re.M):
            names.add(m.group(1))
    return names


def test_header_declares_entry_points():
    names = declared_functions()
    assert {"fadesim_ir_drop_gs_f32", "fadesim_ir_drop_gs_f64", "fadesim_ir_drop_gs_ex",
            "fadesim_last_error"} <= names


def test_library_exports_declared_symbols():
    from fadesim_gb300 import _lib
    from fadesim_gb300.build import build
    build()
    lib = _lib.load()
    for name in declared_functions():
        assert hasattr(lib, name), name
    assert b"sm_103a" in lib.fadesim_version()


def test_argument_errors_without_gpu():
    """Argument checks run before any CUDA call and report like the reference's TORCH_CHECKs."""
    from fadesim_gb300 import _lib
    lib = _lib.load()
    fake = ctypes.c_void_p(16)
    rc = lib.fadesim_ir_drop_gs_f32(fake, fake, 1, 1, 8, 1, 1, 10, 0.34, 1.9, 0, 0.0, 0, None, 0, 0, fake, None)
    assert rc == -1 and b"row_size" in lib.fadesim_last_error()
    rc = lib.fadesim_ir_drop_gs_f32(fake, fake, 1, 8, 8, 1, 1, 10, -1.0, 1.9, 0, 0.0, 0, None, 0, 0, fake, None)
    assert rc == -1 and b"g_wire" in lib.fadesim_last_error()
    rc = lib.fadesim_ir_drop_gs_f32(None, fake, 1, 8, 8, 1, 1, 10, 0.34, 1.9, 0, 0.0, 0, None, 0, 0, fake, None)
    assert rc == -1


def test_host_entry_argument_errors_without_gpu():
    """The host-buffer entry checks its arguments before touching the device;
    an empty batch is a no-op."""
    from fadesim_gb300 import _lib
    lib = _lib.load()
    fake = ctypes.c_void_p(16)
    args = lambda dtype, B, rows, inp, ret_V: (dtype, inp, fake, B, rows, 8, 1, 1, 10, 0.34, 1.9, 0, 0.0, 0, None, 0,
                                               ret_V, fake, None, None, 0, None)
    rc = lib.fadesim_ir_drop_gs_host(*args(7, 1, 8, fake, 0))
    assert rc == -1 and b"dtype" in lib.fadesim_last_error()
    rc = lib.fadesim_ir_drop_gs_host(*args(_lib.F32, 1, 1, fake, 0))
    assert rc == -1 and b"row_size" in lib.fadesim_last_error()
    rc = lib.fadesim_ir_drop_gs_host(*args(_lib.F32, 1, 8, fake, 3))
    assert rc == -1 and b"ret_V" in lib.fadesim_last_error()
    rc = lib.fadesim_ir_drop_gs_host(*args(_lib.F32, 1, 8, None, 0))
    assert rc == -1 and b"null host buffer" in lib.fadesim_last_error()
    assert lib.fadesim_ir_drop_gs_host(*args(_lib.F32, 0, 8, None, 0)) == 0


def test_superposition_refuses_nonlinear_cells():
    from fadesim_gb300 import splitarr
    import pytest as _pt
    with _pt.raises(ValueError):
        splitarr.superposition_solver(splitarr.ArrayConfig(nonlinear_cell_enable=True))


def test_release_memory_without_gpu():
    """Nothing allocated yet: trimming the library's pools is a no-op."""
    from fadesim_gb300 import _lib
    assert _lib.load().fadesim_release_memory() == 0


def _declarations():
    """name -> [parameter kind] of every function include/*.h declares, kinds
    'ptr' or (class, bytes) for scalars."""
    scalars = {"int": ("int", 4), "unsigned int": ("int", 4), "double": ("float", 8), "float": ("float", 4),
               "long long": ("int", 8), "unsigned long long": ("int", 8), "int64_t": ("int", 8),
               "size_t": ("int", 8)}
    out = {}
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        for m in re.finditer(r"\b(fadesim_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", src):
            params = [p.strip() for p in m.group(2).split(",") if p.strip() and p.strip() != "void"]
            kinds = []
            for p in params:
                if "*" in p:
                    kinds.append("ptr")
                    continue
                words = [w for w in p.split() if w != "const"][:-1]  # drop the parameter name
                kinds.append(scalars[" ".join(words)])
            out[m.group(1)] = kinds
    return out


def _kind(t):
    if t is ctypes.c_void_p or hasattr(t, "_type_") and isinstance(t._type_, type):
        return "ptr"
    cls = "float" if t in (ctypes.c_float, ctypes.c_double) else "int"
    return (cls, ctypes.sizeof(t))


def test_ctypes_bindings_match_the_header():
    """Every binding in the ctypes table has the header's parameter count and
    kinds (pointer, integer or floating point of the same width)."""
    from fadesim_gb300 import _lib
    decl = _declarations()
    for name, args in _lib.EXPORTS.items():
        assert name in decl, name
        assert [_kind(t) for t in args] == decl[name], name


def test_warm_start_bindings_match_the_header():
    from fadesim_gb300 import warmstart
    m = {"v": ctypes.c_void_p, "p": ctypes.c_void_p, "i": ctypes.c_int, "l": ctypes.c_longlong, "f": ctypes.c_float}
    decl = _declarations()
    for name, sig in warmstart._SIGS.items():
        assert name in decl, name
        assert [_kind(m[c]) for c in sig] == decl[name], name


def test_every_declared_function_has_a_binding():
    from fadesim_gb300 import _lib, warmstart
    assert set(_declarations()) == set(_lib.EXPORTS) | set(warmstart._SIGS)


def test_constants_match_the_header():
    """The Python side's dtype, method and status codes are the header's #defines."""
    from fadesim_gb300 import _lib
    src = open(os.path.join(ROOT, "include", "fadesim_gb300.h")).read()
    defs = {m.group(1): int(m.group(2)) for m in re.finditer(r"#define\s+FADESIM_([A-Z0-9_]+)\s+\(?(-?\d+)\)?", src)}
    for name in ("F32", "F64", "METHOD_AUTO", "METHOD_LINE", "METHOD_RBSOR", "METHOD_SWEEPS", "METHOD_LINE_COARSE",
                 "ST_CONVERGED", "ST_MAXITER", "ST_NONFINITE", "ST_WARM_REJECTED"):
        assert getattr(_lib, name) == defs[name], name
    from fadesim_gb300 import cpp_ir_drop_accelerate as acc
    assert set(acc._METHODS.values()) == {defs[k] for k in defs if k.startswith("METHOD_")}


def test_header_builds_and_links_from_c(tmp_path):
    """A C99 program includes the header, fills the options struct and links
    against the library (the binding a C, cgo or FFI caller makes); it runs
    without a GPU by asking only for the version string."""
    import shutil
    import subprocess
    from fadesim_gb300.build import build
    if shutil.which("gcc") is None:
        import pytest
        pytest.skip("no C compiler")
    lib = build()
    src = tmp_path / "caller.c"
    src.write_text('#include <stdio.h>\n#include "fadesim_gb300.h"\n'
                   "int main(void) {\n"
                   "    fadesim_solve_opts o = {FADESIM_METHOD_LINE_COARSE, 5e-7, 0, 0, 0.0, 0, 0, 0.0, 0, 0, 1};\n"
                   '    printf("%d %d|%s\\n", o.method, o.fp32_limit, fadesim_version());\n'
                   "    return 0;\n}\n")
    exe = tmp_path / "caller"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), str(src),
                    "-L", os.path.dirname(lib), "-lfadesim_gb300", "-o", str(exe)], check=True, capture_output=True)
    env = dict(os.environ, LD_LIBRARY_PATH=os.path.dirname(lib) + os.pathsep + os.environ.get("LD_LIBRARY_PATH", ""))
    fields, version = subprocess.run([str(exe)], check=True, capture_output=True, text=True,
                                     env=env).stdout.strip().split("|", 1)
    assert fields.split() == ["4", "1"] and "sm_103a" in version


def test_ctypes_structs_match_the_c_layout(tmp_path):
    """The ctypes mirrors of fadesim_solve_opts and fadesim_solve_stats have the
    C compiler's size and field offsets."""
    import shutil
    import subprocess
    from fadesim_gb300 import _lib
    if shutil.which("gcc") is None:
        import pytest
        pytest.skip("no C compiler")
    structs = {"fadesim_solve_opts": _lib.SolveOpts, "fadesim_solve_stats": _lib.SolveStats}
    lines = ['#include <stddef.h>', '#include <stdio.h>', '#include "fadesim_gb300.h"', "int main(void) {"]
    for cname, py in structs.items():
        lines.append('    printf("%s %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('    printf("%s.%s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["    return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), str(src), "-o",
                    str(exe)], check=True, capture_output=True)
    got = dict(line.split() for line in subprocess.run([str(exe)], check=True, capture_output=True,
                                                       text=True).stdout.splitlines())
    for cname, py in structs.items():
        assert int(got[cname]) == ctypes.sizeof(py), cname
        for f, _ in py._fields_:
            assert int(got["%s.%s" % (cname, f)]) == getattr(py, f).offset, (cname, f)
