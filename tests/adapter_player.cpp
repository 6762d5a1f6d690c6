// adapter_player.cpp -- test program: plays a recorded stream of
// PuresoftPipeline calls through the C++ adapter (include/ps3d.hpp, the
// reference's class and method names over the C ABI) and writes what it read
// back, so a test can compare the adapter's output with the oracle's.
//
//   adapter_player <calls.bin> <out.bin>
//
// calls.bin: int32 width, height, then records of int32 opcode + operands
// (layout below, written by tests/test_adapter.py); out.bin: the colour
// buffer (width * height * 4 bytes) after the last call, then the bytes of
// each READ_TEXTURE in order.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <vector>
#include "ps3d.hpp"

namespace {

enum Op : int32_t {
    END = 0, CREATE_TEXTURE = 1, WRITE_LAYER = 2, ADD_PROCESSOR = 3, CREATE_PROGRAMME = 4, USE_PROGRAMME = 5,
    CREATE_VAO = 6, ATTACH_VBO = 7, SET_UNIFORM = 8, SET_DEPTH = 9, SET_VIEWPORT = 10, ENABLE = 11, DISABLE = 12,
    CLEAR_DEPTH = 13, CLEAR_COLOUR = 14, DRAW_VAO = 15, UPDATE_VBO = 16, READ_TEXTURE = 17, POST_PROCESS = 18,
};

struct Reader {
    FILE* f;
    int32_t i32()
    {
        int32_t v;
        if (fread(&v, 4, 1, f) != 1) throw std::runtime_error("truncated call stream");
        return v;
    }
    float f32()
    {
        float v;
        if (fread(&v, 4, 1, f) != 1) throw std::runtime_error("truncated call stream");
        return v;
    }
    std::vector<uint8_t> bytes()
    {
        int64_t n;
        if (fread(&n, 8, 1, f) != 1 || n < 0) throw std::runtime_error("truncated call stream");
        std::vector<uint8_t> b((size_t)n);
        if (n && fread(b.data(), 1, (size_t)n, f) != (size_t)n) throw std::runtime_error("truncated call stream");
        return b;
    }
};

}  // namespace

int main(int argc, char** argv)
{
    if (argc != 3) {
        fprintf(stderr, "usage: %s calls.bin out.bin\n", argv[0]);
        return 2;
    }
    FILE* in = fopen(argv[1], "rb");
    FILE* out = fopen(argv[2], "wb");
    if (!in || !out) return 2;
    try {
        Reader r{in};
        const int w = r.i32(), h = r.i32();
        ps3d_gpu::PuresoftPipeline pipe(w, h);
        std::vector<uint8_t> reads;
        for (;;) {
            const int32_t op = r.i32();
            if (op == END) break;
            switch (op) {
            case CREATE_TEXTURE: {
                ps3d_gpu::ImageBuffer img;
                img.width = (unsigned)r.i32();
                img.height = (unsigned)r.i32();
                img.scanline = (unsigned)r.i32();
                img.elemLen = (unsigned)r.i32();
                const int wrap = r.i32(), extra = r.i32();
                std::vector<uint8_t> px = r.bytes();
                img.pixels = px.empty() ? nullptr : px.data();
                pipe.createTexture(&img, extra, wrap != 0);
                break;
            }
            case WRITE_LAYER: {
                const int idx = r.i32(), layer = r.i32();
                std::vector<uint8_t> px = r.bytes();
                pipe.writeTexture(idx, px.data(), px.size(), layer);
                break;
            }
            case ADD_PROCESSOR: pipe.addProcessor(r.i32()); break;
            case CREATE_PROGRAMME: {
                const int v = r.i32(), i = r.i32(), f = r.i32();
                pipe.createProgramme(v, i, f);
                break;
            }
            case USE_PROGRAMME: pipe.useProgramme(r.i32()); break;
            case CREATE_VAO: pipe.createVAO(); break;
            case ATTACH_VBO: {
                const int vao = r.i32(), slot = r.i32(), unit = r.i32(), count = r.i32();
                std::vector<uint8_t> data = r.bytes();
                pipe.attachVBO(vao, slot, unit, count, data.data());
                break;
            }
            case UPDATE_VBO: {  // the demo's getVBO(vao, idx)->updateContent(src) (test/scenobj.cpp:135-157)
                const int vao = r.i32(), slot = r.i32();
                std::vector<uint8_t> data = r.bytes();
                pipe.getVBO(vao, slot).updateContent(data.data());
                break;
            }
            case SET_UNIFORM: {
                const int idx = r.i32();
                std::vector<uint8_t> data = r.bytes();
                pipe.setUniform(idx, data.data(), data.size());
                break;
            }
            case SET_DEPTH: pipe.setDepth(r.i32()); break;
            case SET_VIEWPORT: {
                const int vw = r.i32(), vh = r.i32();
                pipe.setViewport(vw, vh);
                break;
            }
            case ENABLE: pipe.enable(r.i32()); break;
            case DISABLE: pipe.disable(r.i32()); break;
            case CLEAR_DEPTH: pipe.clearDepth(r.f32()); break;
            case CLEAR_COLOUR: pipe.clearColour((uint32_t)r.i32()); break;
            case DRAW_VAO: pipe.drawVAO(r.i32()); break;
            case POST_PROCESS: {
                const int id = r.i32();
                std::vector<uint8_t> params = r.bytes();
                pipe.postProcess(id, params.empty() ? nullptr : params.data(), params.size());
                break;
            }
            case READ_TEXTURE: {
                const int idx = r.i32();
                const int64_t n = (int64_t)r.i32() * r.i32();  // scanline x height
                std::vector<uint8_t> buf((size_t)n);
                pipe.readTexture(idx, buf.data(), buf.size());
                reads.insert(reads.end(), buf.begin(), buf.end());
                break;
            }
            default: throw std::runtime_error("unknown call in the stream");
            }
        }
        std::vector<uint8_t> frame((size_t)w * h * 4);
        pipe.readColour(frame.data());
        fwrite(frame.data(), 1, frame.size(), out);
        if (!reads.empty()) fwrite(reads.data(), 1, reads.size(), out);
    } catch (const std::exception& e) {
        fprintf(stderr, "adapter_player: %s\n", e.what());
        return 1;
    }
    fclose(in);
    fclose(out);
    return 0;
}
