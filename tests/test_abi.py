"""CPU checks of the C ABI: the library loads and exports every entry point
that include/fs3d.h declares, the ctypes binding's signatures and structs
match the header, its host-side generators match the oracle's, and bad
arguments come back as status codes (no GPU work is issued here)."""
import ctypes as C
import os
import re

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    txt = open(os.path.join(ROOT, "include", "fs3d.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(fs3d_[a-z0-9_]+)\s*\(", txt)))


def test_header_and_binding_agree(fs3d):
    assert declared_functions() == sorted(fs3d.EXPORTS)


def test_library_exports_every_declared_symbol(fs3d):
    L = fs3d.lib()
    for name in declared_functions():
        assert hasattr(L, name), name
    assert L.fs3d_abi_version() == 1
    assert L.fs3d_status_string(-3) == b"over the memory budget"


def test_struct_layouts_match_header(fs3d, tmp_path):
    """Every struct of the binding has the header's size and field offsets:
    a C program compiled against include/fs3d.h prints them (gcc, no GPU)."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    structs = {"fs3d_camera": fs3d.Camera, "fs3d_config": fs3d.Config, "fs3d_world_spec": fs3d.WorldSpec,
               "fs3d_tune_report": fs3d.TuneReport, "fs3d_serve_params": fs3d.ServeParams,
               "fs3d_serve_request": fs3d.ServeRequest, "fs3d_serve_stats": fs3d.ServeStats,
               "fs3d_object_view": fs3d.ObjectView, "fs3d_mesh_draw": fs3d.MeshDraw}
    cname = lambda f: "lambda" if f == "lambda_" else f  # a Python keyword renamed in the binding
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "fs3d.h"', "int main(void) {"]
    for s, cls in structs.items():
        lines.append(f'    printf("{s} size %zu\\n", sizeof({s}));')
        for f, _ in cls._fields_:
            lines.append(f'    printf("{s} {f} %zu\\n", offsetof({s}, {cname(f)}));')
    lines += ["    return 0;", "}"]
    src, exe = tmp_path / "layout.c", tmp_path / "layout"
    src.write_text("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    got = {}
    for ln in subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.splitlines():
        s, f, v = ln.split()
        got[(s, f)] = int(v)
    for s, cls in structs.items():
        assert got[(s, "size")] == C.sizeof(cls), s
        for f, _ in cls._fields_:
            assert got[(s, f)] == getattr(cls, f).offset, (s, f)
    # the numpy view used to build many world specs at once
    for f in fs3d._SPEC_DTYPE.names:
        assert fs3d._SPEC_DTYPE.fields[f][1] == got[("fs3d_world_spec", f)], f
    assert fs3d._SPEC_DTYPE.itemsize == got[("fs3d_world_spec", "size")]


def header_declarations():
    """(return type, name, [parameter declarations]) of every function in include/fs3d.h."""
    txt = open(os.path.join(ROOT, "include", "fs3d.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    txt = re.sub(r"^\s*#.*$", "", txt, flags=re.M)
    out = []
    for ret, name, params in re.findall(r"([A-Za-z_][\w \t\*]*?)\b(fs3d_\w+)\s*\(([^;{()]*)\)\s*;", txt):
        ps = [p.strip() for p in " ".join(params.split()).split(",")]
        out.append((" ".join(ret.split()), name, [] if ps == ["void"] else ps))
    return out


def test_binding_signatures_match_header(fs3d, tmp_path):
    """Each function's ctypes signature agrees with its C prototype: the
    parameter count, pointer or value for each parameter, the value widths
    (sizes from a gcc-compiled probe), the struct a pointer points to, and
    the return type."""
    import shutil
    import subprocess
    if not shutil.which("gcc"):
        pytest.skip("gcc not found")
    structs = {"fs3d_camera": fs3d.Camera, "fs3d_config": fs3d.Config, "fs3d_world_spec": fs3d.WorldSpec,
               "fs3d_tune_report": fs3d.TuneReport, "fs3d_serve_params": fs3d.ServeParams,
               "fs3d_serve_request": fs3d.ServeRequest, "fs3d_serve_stats": fs3d.ServeStats,
               "fs3d_object_view": fs3d.ObjectView, "fs3d_mesh_draw": fs3d.MeshDraw}
    decls = header_declarations()
    assert sorted(n for _, n, _ in decls) == declared_functions()

    def split(p):  # "const uint8_t* grid" -> ("const uint8_t*", pointer?)
        if "*" in p:
            return p[:p.rindex("*") + 1], True
        toks = p.split()
        return " ".join(toks[:-1]), False

    value_types = sorted({split(p)[0] for _, _, ps in decls for p in ps if not split(p)[1]})
    src = tmp_path / "sizes.c"
    src.write_text('#include <stdio.h>\n#include "fs3d.h"\nint main(void) {\n' +
                   "".join(f'    printf("{t}=%zu\\n", sizeof({t}));\n' for t in value_types) + "    return 0;\n}\n")
    exe = tmp_path / "sizes"
    subprocess.run(["gcc", "-std=c11", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)], check=True)
    size = dict(ln.split("=") for ln in subprocess.run([str(exe)], capture_output=True, text=True,
                                                       check=True).stdout.split())
    pointer_types = (C.c_void_p, C.c_char_p)
    rets = {"fs3d_status": C.c_int, "int": C.c_int, "const char*": C.c_char_p, "uint64_t": C.c_uint64,
            "fs3d_config": fs3d.Config, "void": None}
    L = fs3d.lib()
    for ret, name, params in decls:
        fn = getattr(L, name)
        assert fn.restype is rets[ret], (name, ret)
        assert len(fn.argtypes) == len(params), name
        for p, at in zip(params, fn.argtypes):
            ctype, is_ptr = split(p)
            if is_ptr:
                assert at in pointer_types or issubclass(at, C._Pointer), (name, p, at)
                base = ctype.replace("const", "").replace("*", "").strip()
                if base in structs and ctype.count("*") == 1:
                    assert at is C.c_void_p or at._type_ is structs[base], (name, p, at)
            else:
                assert at not in pointer_types and not issubclass(at, C._Pointer), (name, p, at)
                assert C.sizeof(at) == int(size[ctype]), (name, p, at)


def test_integration_binding_compiles_against_the_header(tmp_path):
    """The C++ binding that the integration guide shows a maintainer adding
    to the engine type-checks against include/fs3d.h (g++ -fsyntax-only, the
    engine's own names stubbed)."""
    import shutil
    import subprocess
    if not shutil.which("g++"):
        pytest.skip("g++ not found")
    txt = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    blocks = re.findall(r"```cpp\n(.*?)```", txt, flags=re.S)
    assert len(blocks) == 1
    body = "\n".join(ln for ln in blocks[0].splitlines() if not ln.startswith("#include"))
    src = tmp_path / "binding.cpp"
    src.write_text('#include <cstdint>\n#include <vector>\n#include "fs3d.h"\n'
                   "namespace util { inline void displayError(const char*) {} }\n"
                   "struct Vec3 { float x, y, z; };\n"
                   "static Vec3 camPos, camRot;\n"
                   "static float *frameDevPtr, *objectFrameDevPtr;\n"
                   "void engine_hooks() {\n" + body + "\n}\n")
    r = subprocess.run(["g++", "-std=c++17", "-fsyntax-only", "-Wall", "-Wno-unused-variable",
                        "-I", os.path.join(ROOT, "include"), str(src)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_default_config(fs3d):
    c = fs3d.lib().fs3d_default_config()
    assert c.steps_per_segment == 64 and c.use_graphs == 1


def test_generators_match_oracle(fs3d, orc):
    for seed in (1, 2):
        assert (fs3d.gen_parity(seed) == orc.gen_c1(seed)).all()
    assert (fs3d.gen_pillars(3, 96, 128, 80) == orc.gen_c2(3, 96, 128, 80)).all()
    assert (fs3d.gen_dunes(4, 96, 80, 64) == orc.gen_c5(4, 96, 80, 64)).all()
    d1, s1 = fs3d.gen_batch_dims(9, 64)
    d2, s2 = orc.gen_c3_dims(9, 64)
    assert (d1 == d2).all() and (s1 == s2).all()
    for w in range(3):
        X, Y, Z = (int(v) for v in d1[w])
        assert (fs3d.gen_batch_world(int(s1[w]), X, Y, Z) == orc.gen_c3_world(int(s2[w]), X, Y, Z)).all()


def test_camera_presets(fs3d):
    c = fs3d.camera_fs_raymarch()
    assert list(c.origin) == [0.0, 0.0, -5.0] and abs(c.aspect - 1700 / 900) < 1e-6
    assert list(c.light_pos) == [2.0, 5.0, 3.0]
    v = fs3d.camera_world_view(1024, 1024, 1024, 1920, 1080)
    f = np.array(v.forward)
    assert abs(np.linalg.norm(f) - 1) < 1e-6 and abs(v.tan_half_fov - np.tan(np.radians(35))) < 1e-6


def test_bad_arguments_return_status(fs3d):
    L = fs3d.lib()
    h = C.c_void_p()
    g = np.zeros(8, np.uint8)
    assert L.fs3d_world_create(None, 2, 2, 2, 0, 0, 0, C.byref(h)) == fs3d.ERR_INVALID_ARG
    assert L.fs3d_world_create(g.ctypes.data, 0, 2, 2, 0, 0, 0, C.byref(h)) == fs3d.ERR_INVALID_ARG
    assert L.fs3d_world_create(g.ctypes.data, 2, 2, 2, 0, 0, 7, C.byref(h)) == fs3d.ERR_INVALID_ARG
    assert b"layout" in L.fs3d_last_error()
    assert L.fs3d_step_device(None, 2, 2, 2, 0, 0, 1, None) == fs3d.ERR_INVALID_ARG
    assert L.fs3d_world_step(None, 1) == fs3d.ERR_INVALID_ARG
    assert L.fs3d_world_destroy(None) == fs3d.ERR_INVALID_ARG
    assert L.fs3d_batch_admit(None, None, 1, 1, 1, 0, 0, 1, None) == fs3d.ERR_INVALID_ARG
    assert L.fs3d_gen_parity(1, 0, 4, 4, g.ctypes.data) == fs3d.ERR_INVALID_ARG
    with pytest.raises(fs3d.Fs3dError) as e:
        fs3d.check(fs3d.ERR_BUDGET)
    assert e.value.status == fs3d.ERR_BUDGET
    assert L.fs3d_world_load(b"/nonexistent/ckp", 0, C.byref(h)) == fs3d.ERR_IO


# every entry point that takes a handle or a required pointer, with it NULL:
# refused on the host with FS3D_ERR_INVALID_ARG (no CUDA call, no crash)
NULL_CALLS = {
    "fs3d_world_step": (None, 1), "fs3d_world_sync": (None, 0), "fs3d_world_read": (None, None),
    "fs3d_world_write": (None, None), "fs3d_world_hash": (None, None), "fs3d_world_device_ptr": (None, None, None),
    "fs3d_world_stream": (None, None), "fs3d_world_destroy": (None,), "fs3d_world_save": (None, b"ckp"),
    "fs3d_world_info": (None, None, None, None, None, None, None),
    "fs3d_world_create": (None, 2, 2, 2, 0, 0, 0, None), "fs3d_world_load": (None, 0, None),
    "fs3d_batch_create": (0, None, None),
    "fs3d_batch_admit": (None, None, 1, 1, 1, 0, 0, 1, None),
    "fs3d_batch_admit_generated": (None, 16, 16, 16, 0, 0, 1, None),
    "fs3d_batch_admit_many": (None, 1, None, None, None), "fs3d_batch_admit_many_async": (None, 1, None, None, None),
    "fs3d_batch_run_segment": (None,), "fs3d_batch_prepare": (None,), "fs3d_batch_sync": (None, 0),
    "fs3d_batch_poll": (None, 1, None, None), "fs3d_batch_poll_many": (None, 1, None, None, None),
    "fs3d_batch_retire": (None, 1, None), "fs3d_batch_retire_many": (None, 1, None, None),
    "fs3d_batch_retire_many_async": (None, 1, None, None), "fs3d_batch_read_many": (None, 1, None, None),
    "fs3d_batch_wait_copies": (None, 0), "fs3d_batch_autotune": (None, 1, None),
    "fs3d_batch_counters": (None, None, None), "fs3d_batch_stream": (None, None), "fs3d_batch_destroy": (None,),
    "fs3d_batch_stats": (None, None, None, None, None),
    "fs3d_step_device": (None, 2, 2, 2, 0, 0, 1, None), "fs3d_step_device_many": (1, None, None, None, 0, 1, None),
    "fs3d_run_device": (None, 2, 2, 2, 0, 0, 1, None), "fs3d_run_device_noalloc": (None, 2, 2, 2, 0, 0, 1, None),
    "fs3d_serve_plan": (None, 0, None, None), "fs3d_serve_run": (None, 0, None, None),
    "fs3d_render": (None, None, 16, 16, 0, None, 0), "fs3d_render_sdf": (None, 16, 16, None, None),
}


@pytest.mark.parametrize("name", sorted(NULL_CALLS))
def test_null_handles_and_pointers_are_refused(fs3d, name):
    L = fs3d.lib()
    assert getattr(L, name)(*NULL_CALLS[name]) == fs3d.ERR_INVALID_ARG
    assert L.fs3d_last_error() != b""


def test_object_render_rejects_before_launch(fs3d):
    """Views the restatement does not cover are refused on the host, with no
    device work: an eye inside the cube (a vertex behind the camera), a
    singular model, and more than 48 triangles."""
    tri = fs3d.mesh_cube()
    fake = 16  # never dereferenced: every case fails in the host set-up
    for view in (fs3d.object_view_scene(cam_pos=(0.0, 0.0, 0.0)),
                 fs3d.object_view_scene(model=np.zeros((4, 4)))):
        with pytest.raises(fs3d.Fs3dError) as e:
            fs3d.render_object_device(view, tri, 64, 32, fake)
        assert e.value.status == fs3d.ERR_INVALID_ARG
    with pytest.raises(fs3d.Fs3dError):
        fs3d.render_object_device(fs3d.object_view_scene(), np.concatenate([tri] * 5), 64, 32, fake)
    assert fs3d.mesh_cube().shape == (12, 3, 3)


def test_no_cpu_fallback_without_a_gpu(fs3d):
    """The product library has no CPU path for the step: on a machine with no
    usable GPU, creating a world or a batch fails with FS3D_ERR_CUDA instead
    of stepping on the host."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    g = fs3d.gen_parity(1)
    with pytest.raises(fs3d.Fs3dError) as e:
        fs3d.World(g, 1)
    assert e.value.status == fs3d.ERR_CUDA
    with pytest.raises(fs3d.Fs3dError) as e:
        fs3d.Batch(1 << 30)
    assert e.value.status == fs3d.ERR_CUDA
