"""The C ABI: the CUDA library loads and exports every entry point
include/ps3d.h declares (no device calls)."""
import os
import re
import subprocess

from puresoft3d_gb300 import build, pipeline

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    names = set()
    for h in [f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")]:
        txt = open(os.path.join(ROOT, "include", h)).read()
        names |= set(re.findall(r"^\s*(?:const\s+)?\w[\w\s\*]*?\b(ps3d_\w+)\s*\(", txt, re.M))
    return names


def test_header_declares_entry_points():
    d = declared()
    assert "ps3d_draw" in d and "ps3d_pipeline_create" in d and len(d) >= 30


def test_library_exports_every_declared_symbol():
    lib = build.build()
    out = subprocess.run(["nm", "-D", "--defined-only", lib], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\bT (ps3d_\w+)", out))
    missing = declared() - exported
    assert not missing, missing


def test_python_binding_covers_header():
    assert declared() <= set(pipeline.exported_symbols()) | {"ps3d_last_error"}


def test_library_loads():
    lib = pipeline.library()
    assert lib.ps3d_last_error() is not None


def test_cpp_adapter_compiles(tmp_path):
    """include/ps3d.hpp (the reference's class and method names over the C
    ABI) compiles and links against the library (no device calls)."""
    src = tmp_path / "use_adapter.cpp"
    src.write_text('''
#include "ps3d.hpp"
int main(int argc, char**) {
    if (argc > 5) {  // never taken: only the calls' types are checked
        ps3d_gpu::PuresoftPipeline pipe(64, 48);
        ps3d_gpu::ImageBuffer img = {4, 16, 4, 4, nullptr};
        int cube = pipe.createTexture(&img, 5);
        pipe.writeTexture(cube, nullptr, 0, 3);
        int prog = pipe.createProgramme(pipe.addProcessor(PS3D_VP_DEF04), pipe.addProcessor(PS3D_IP_DEF04),
                                        pipe.addProcessor(PS3D_FP_DEF04));
        pipe.useProgramme(prog);
        int vao = pipe.createVAOFromObjx("sphere.objx");
        pipe.getVBO(vao, 0).updateContent(nullptr);
        pipe.drawVAO(vao);
        pipe.postProcess(PS3D_PP_ADD8);
        unsigned char frame[64 * 48 * 4];
        pipe.readColour(frame);
    }
    return 0;
}
''')
    lib = build.build()
    out = tmp_path / "use_adapter"
    subprocess.run(["g++", "-std=c++17", "-I", os.path.join(ROOT, "include"), str(src), lib, "-o", str(out)],
                   check=True, capture_output=True, text=True)
    assert out.exists()
