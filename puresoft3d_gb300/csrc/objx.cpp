// objx.cpp -- the reference's OBJX mesh container (src/objcvt/objxio.h:42-52,
// objxio.cpp): a file header (version 0x010003, mesh count, mesh-header
// size, camera and four lights) and, per mesh, a packed 1627-byte header
// followed by float4 positions, float4 normals, float4 tangents, float2
// texture coordinates (each present as the header says) and int32 indices.
// All little-endian, as the reference writes it on x86; read and written
// here field by field, so the same code serves x86-64 and AArch64 hosts.
//
// ps3d_objx_load_vao builds the vertex arrays the reference demo builds from
// an OBJX mesh (src/test/scenobj.cpp:88-162) straight into a pipeline's VAO:
// slot 0 positions with w = 1, 1 tangents, 2 binormals = normalise(cross(
// normal, tangent)), 3 normals, 4 texture coordinates -- the layout of the
// reference's bump-mapped processors (DEF03).
#include <stdio.h>
#include <string.h>
#include <math.h>
#include <vector>
#include "ps3d.h"
#include "ps3d_internal.h"

using ps3d::report_error;

namespace {

constexpr unsigned kObjxVersion = 0x010003;  // objxio.cpp:6
constexpr int kName = 260;                   // OBJX_FILENAMELEN
constexpr int kFileHeader = 16 + 16 + 16 + 4 * 32;
constexpr int kMeshHeader = kName + 4 + 4 + 3 + 3 * 16 + 4 + 5 * kName + 4;  // 1627, #pragma pack(1)

struct Buf {
    std::vector<unsigned char> b;
    size_t at = 0;
    void u32(unsigned v)
    {
        for (int k = 0; k < 4; k++) b.push_back((unsigned char)(v >> (8 * k)));
    }
    void f32(float f)
    {
        unsigned v;
        memcpy(&v, &f, 4);
        u32(v);
    }
    void bytes(const void* p, size_t n) { b.insert(b.end(), (const unsigned char*)p, (const unsigned char*)p + n); }
    void str(const char* s)
    {
        char tmp[kName] = {};
        if (s) strncpy(tmp, s, kName - 1);
        bytes(tmp, kName);
    }
    unsigned ru32()
    {
        unsigned v = 0;
        for (int k = 0; k < 4; k++) v |= (unsigned)b[at + k] << (8 * k);
        at += 4;
        return v;
    }
    float rf32()
    {
        unsigned v = ru32();
        float f;
        memcpy(&f, &v, 4);
        return f;
    }
    void rstr(char* out)
    {
        memcpy(out, &b[at], kName);
        out[kName - 1] = 0;
        at += kName;
    }
};

float clamp01(float v) { return v < 0.0f ? 0.0f : (v > 1.0f ? 1.0f : v); }

// 4-lane mcemaths operations, IEEE where the reference uses rsqrtss
void sub4(float* r, const float* a, const float* b)
{
    for (int k = 0; k < 4; k++) r[k] = a[k] - b[k];
}
void norm4(float* v)  // mcemaths_norm_3_4 (vector.cpp:225-250): v * 1/sqrt(haddps(v*v))
{
    float s = (v[0] * v[0] + v[1] * v[1]) + (v[2] * v[2] + v[3] * v[3]);
    float r = 1.0f / sqrtf(s);
    for (int k = 0; k < 4; k++) v[k] = v[k] * r;
}
void cross3(float* r, const float* a, const float* b)  // mcemaths_cross_3 (vector.cpp:114-144), lane 3 a3*b3 - a3*b3
{
    float o[4] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0], a[3] * b[3] - a[3] * b[3]};
    memcpy(r, o, 16);
}

// generate_tangent (objxio.cpp:445-471) as it is evidently meant: the
// reference overwrites its first edge vector with the second and reads an
// uninitialised one, so its result is undefined; here v1 = c - a,
// v2 = b - a, tangent = (v1 * dv2 - v2 * dv1) / (du1 * dv2 - dv1 * du2).
void gen_tangent(float* t, const float* a, const float* b, const float* c, const float* ta, const float* tb,
                 const float* tc)
{
    float du1 = tc[0] - ta[0], dv1 = tc[1] - ta[1], du2 = tb[0] - ta[0], dv2 = tb[1] - ta[1];
    float v1[4], v2[4];
    sub4(v1, c, a);
    sub4(v2, b, a);
    for (int k = 0; k < 4; k++) v1[k] = v1[k] * dv2;
    for (int k = 0; k < 4; k++) v2[k] = v2[k] * dv1;
    sub4(t, v1, v2);
    float f = 1.0f / (du1 * dv2 - dv1 * du2);
    for (int k = 0; k < 4; k++) t[k] = t[k] * f;
}

}  // namespace

struct ps3d_objx {
    FILE* f = nullptr;
    bool writing = false;
    unsigned meshes = 0, meshHeaderSize = kMeshHeader;
    std::vector<unsigned char> header;  // the file header as read or to be written
    ps3d_objx_mesh_info last = {};
    long meshStart = 0;  // file offset of the last mesh's data
    unsigned nextOffset = 0;
};

extern "C" {

int ps3d_objx_create(const char* path, const ps3d_objx_scene* scn, ps3d_objx** out)
{
    if (!path || !scn || !out) return report_error(PS3D_ERR_INVALID, "null argument");
    ps3d_objx* h = new ps3d_objx();
    h->f = fopen(path, "w+b");
    if (!h->f) {
        delete h;
        return report_error(PS3D_ERR_INVALID, "cannot create the OBJX file");
    }
    h->writing = true;
    Buf b;
    b.u32(kObjxVersion);
    b.u32(0);
    b.u32(kMeshHeader);
    b.u32(0);
    for (int k = 0; k < 4; k++) b.f32(scn->camera_pos[k]);
    for (int k = 0; k < 4; k++) b.f32(scn->camera_ypr[k]);
    for (int l = 0; l < 4; l++) {
        for (int k = 0; k < 4; k++) b.f32(scn->light_pos[l][k]);
        for (int k = 0; k < 4; k++) b.f32(scn->light_dir[l][k]);
    }
    h->header = b.b;
    fwrite(h->header.data(), 1, h->header.size(), h->f);
    *out = h;
    return 0;
}

int ps3d_objx_write_mesh(ps3d_objx* h, const ps3d_objx_mesh_info* m, const float* vertices, const float* normals,
                         const float* tangents, const float* texcoords, const int* indices)
{
    if (!h || !m || !h->writing) return report_error(PS3D_ERR_INVALID, "not an OBJX file open for writing");
    // write_mesh (objxio.cpp:98-181): vertices required; indices iff num_indices
    if (m->num_vertices == 0 || !vertices || (m->num_indices != 0) != (indices != nullptr))
        return report_error(PS3D_ERR_INVALID, "write_mesh: missing vertices or indices");
    const unsigned nv = m->num_vertices, ni = m->num_indices;
    unsigned bytes = nv * 16 + (texcoords ? nv * 8 : 0) + (normals ? nv * 16 : 0) + (tangents ? nv * 16 : 0) + ni * 4;
    Buf b;
    b.str(m->name);
    b.u32(nv);
    b.u32(ni);
    unsigned char has[3] = {(unsigned char)(texcoords != nullptr), (unsigned char)(normals != nullptr),
                            (unsigned char)(tangents != nullptr)};
    b.bytes(has, 3);
    // colours are stored b, g, r, a (objxio.cpp:121-132)
    const float* cols[3] = {m->ambient, m->diffuse, m->specular};
    for (const float* c : cols) {
        b.f32(c[2]);
        b.f32(c[1]);
        b.f32(c[0]);
        b.f32(c[3]);
    }
    b.f32(m->specular_exponent);
    b.str(m->diffuse_file);
    b.str(m->bump_file);
    b.str(m->spc_file);
    b.str(m->spe_file);
    b.str(m->programme);
    b.u32(bytes);  // next_offset (calc_mesh_bytes, objxio.cpp:383-396)
    for (unsigned i = 0; i < 4 * nv; i++) b.f32(vertices[i]);
    if (normals)
        for (unsigned i = 0; i < 4 * nv; i++) b.f32(normals[i]);
    if (tangents)
        for (unsigned i = 0; i < 4 * nv; i++) b.f32(tangents[i]);
    if (texcoords)
        for (unsigned i = 0; i < 2 * nv; i++) b.f32(texcoords[i]);
    for (unsigned i = 0; i < ni; i++) b.u32((unsigned)indices[i]);
    if (fwrite(b.b.data(), 1, b.b.size(), h->f) != b.b.size()) return report_error(PS3D_ERR_INVALID, "write failed");
    h->meshes++;
    return 0;
}

int ps3d_objx_open(const char* path, ps3d_objx_scene* scn, ps3d_objx** out)
{
    if (!path || !out) return report_error(PS3D_ERR_INVALID, "null argument");
    FILE* f = fopen(path, "rb");
    if (!f) return report_error(PS3D_ERR_INVALID, "cannot open the OBJX file");
    Buf b;
    b.b.resize(kFileHeader);
    if (fread(b.b.data(), 1, kFileHeader, f) != (size_t)kFileHeader) {
        fclose(f);
        return report_error(PS3D_ERR_INVALID, "short OBJX file header");
    }
    unsigned version = b.ru32(), meshes = b.ru32(), mhs = b.ru32();
    b.ru32();
    // open_objxW (objxio.cpp:185-226): version and header size checked
    if (version != kObjxVersion || mhs < (unsigned)kMeshHeader) {
        fclose(f);
        return report_error(PS3D_ERR_INVALID, "not an OBJX 1.0.3 file");
    }
    ps3d_objx_scene s = {};
    for (int k = 0; k < 4; k++) s.camera_pos[k] = b.rf32();
    for (int k = 0; k < 4; k++) s.camera_ypr[k] = b.rf32();
    for (int l = 0; l < 4; l++) {
        for (int k = 0; k < 4; k++) s.light_pos[l][k] = b.rf32();
        for (int k = 0; k < 4; k++) s.light_dir[l][k] = b.rf32();
        // a direction of length below 1e-7 marks an omni light (objxio.cpp:212-218)
        const float* d = s.light_dir[l];
        float len = sqrtf((d[0] * d[0] + d[1] * d[1]) + (d[2] * d[2] + d[3] * d[3]));
        s.light_types[l] = len < 0.0000001f ? 0 : 1;
    }
    if (scn) *scn = s;
    ps3d_objx* h = new ps3d_objx();
    h->f = f;
    h->meshes = meshes;
    h->meshHeaderSize = mhs;
    h->header = b.b;
    *out = h;
    return 0;
}

int ps3d_objx_mesh_count(ps3d_objx* h)
{
    if (!h) return report_error(PS3D_ERR_INVALID, "null handle");
    return (int)h->meshes;
}

int ps3d_objx_read_mesh_header(ps3d_objx* h, ps3d_objx_mesh_info* m)
{
    if (!h || !m || h->writing) return report_error(PS3D_ERR_INVALID, "not an OBJX file open for reading");
    Buf b;
    b.b.resize(kMeshHeader);
    if (fread(b.b.data(), 1, kMeshHeader, h->f) != (size_t)kMeshHeader)
        return report_error(PS3D_ERR_RANGE, "no further mesh header");
    // read_mesh_header (objxio.cpp:235-289): a newer, larger header's tail is skipped
    fseek(h->f, (long)(h->meshHeaderSize - kMeshHeader), SEEK_CUR);
    ps3d_objx_mesh_info r = {};
    b.rstr(r.name);
    r.num_vertices = b.ru32();
    r.num_indices = b.ru32();
    r.has_texcoords = b.b[b.at] != 0;
    r.has_normals = b.b[b.at + 1] != 0;
    r.has_tangents = b.b[b.at + 2] != 0;
    b.at += 3;
    float* cols[3] = {r.ambient, r.diffuse, r.specular};
    for (float* c : cols) {  // stored b, g, r, a; returned r, g, b, a clamped to [0, 1]
        float bb = b.rf32(), gg = b.rf32(), rr = b.rf32(), aa = b.rf32();
        c[0] = clamp01(rr);
        c[1] = clamp01(gg);
        c[2] = clamp01(bb);
        c[3] = clamp01(aa);
    }
    r.specular_exponent = b.rf32();
    b.rstr(r.diffuse_file);
    b.rstr(r.bump_file);
    b.rstr(r.spc_file);
    b.rstr(r.spe_file);
    b.rstr(r.programme);
    h->nextOffset = b.ru32();
    h->last = r;
    h->meshStart = ftell(h->f);
    *m = r;
    return 0;
}

int ps3d_objx_read_mesh(ps3d_objx* h, float* vertices, float* normals, float* tangents, float* texcoords,
                        int* indices)
{
    if (!h || h->writing) return report_error(PS3D_ERR_INVALID, "not an OBJX file open for reading");
    const ps3d_objx_mesh_info& m = h->last;
    const size_t nv = m.num_vertices, ni = m.num_indices;
    auto part = [&](bool present, float* dst, size_t floats) -> bool {
        if (!present) return true;
        std::vector<unsigned char> raw(floats * 4);
        if (fread(raw.data(), 1, raw.size(), h->f) != raw.size()) return false;
        if (dst) {
            Buf b;
            b.b.swap(raw);
            for (size_t i = 0; i < floats; i++) dst[i] = b.rf32();
        }
        return true;
    };
    // read_mesh (objxio.cpp:291-368): positions, normals, tangents,
    // texture coordinates, indices, each skipped when not wanted
    bool ok = part(true, vertices, 4 * nv) && part(m.has_normals, normals, 4 * nv) &&
              part(m.has_tangents, m.has_tangents ? tangents : nullptr, 4 * nv) &&
              part(m.has_texcoords, texcoords, 2 * nv);
    if (ok && ni) {
        std::vector<unsigned char> raw(ni * 4);
        ok = fread(raw.data(), 1, raw.size(), h->f) == raw.size();
        if (ok && indices) {
            Buf b;
            b.b.swap(raw);
            for (size_t i = 0; i < ni; i++) indices[i] = (int)b.ru32();
        }
    }
    if (!ok) return report_error(PS3D_ERR_INVALID, "truncated OBJX mesh");
    // tangents asked for, absent in the file, derivable from the texture
    // coordinates (objxio.cpp:336-340, 398-443)
    if (tangents && !m.has_tangents && m.has_texcoords && texcoords && vertices) {
        float t[4];
        if (ni) {
            for (size_t i = 0; i < ni; i++)
                if (indices == nullptr || indices[i] < 0 || (size_t)indices[i] >= nv)
                    return report_error(PS3D_ERR_RANGE, "index out of range");
            // the reference zeroes the positions here (its loop clears
            // mesh.vertices, objxio.cpp:402-411); the tangent sums are meant
            memset(tangents, 0, nv * 16);
            for (size_t i = 0; i + 2 < ni; i += 3) {
                int a = indices[i], bb = indices[i + 1], c = indices[i + 2];
                gen_tangent(t, vertices + 4 * a, vertices + 4 * bb, vertices + 4 * c, texcoords + 2 * a,
                            texcoords + 2 * bb, texcoords + 2 * c);
                for (int k = 0; k < 4; k++) {
                    tangents[4 * a + k] += t[k];
                    tangents[4 * bb + k] += t[k];
                    tangents[4 * c + k] += t[k];
                }
            }
            for (size_t i = 0; i < nv; i++) norm4(tangents + 4 * i);
        } else {
            for (size_t i = 0; i + 2 < nv; i += 3) {
                gen_tangent(t, vertices + 4 * i, vertices + 4 * (i + 1), vertices + 4 * (i + 2), texcoords + 2 * i,
                            texcoords + 2 * (i + 1), texcoords + 2 * (i + 2));
                norm4(t);
                for (int v = 0; v < 3; v++) memcpy(tangents + 4 * (i + v), t, 16);
            }
        }
    }
    fseek(h->f, h->meshStart, SEEK_SET);
    fseek(h->f, (long)h->nextOffset, SEEK_CUR);
    return 0;
}

int ps3d_objx_close(ps3d_objx* h)
{
    if (!h) return 0;
    if (h->writing) {  // close_objx (objxio.cpp:370-381): the mesh count goes into the header
        Buf b;
        b.u32(h->meshes);
        fseek(h->f, 4, SEEK_SET);
        fwrite(b.b.data(), 1, 4, h->f);
    }
    fclose(h->f);
    delete h;
    return 0;
}

int ps3d_objx_load_vao(ps3d_pipeline* p, const char* path, int meshIndex, int* vaoOut)
{
    if (!p || !path || !vaoOut) return report_error(PS3D_ERR_INVALID, "null argument");
    ps3d_objx* h = nullptr;
    int rc = ps3d_objx_open(path, nullptr, &h);
    if (rc) return rc;
    ps3d_objx_mesh_info m;
    for (int i = 0; i <= meshIndex && !rc; i++) {
        if (i >= (int)h->meshes) rc = report_error(PS3D_ERR_RANGE, "the OBJX file has fewer meshes");
        else if (!(rc = ps3d_objx_read_mesh_header(h, &m)) && i < meshIndex) rc = ps3d_objx_read_mesh(h, 0, 0, 0, 0, 0);
    }
    if (rc) {
        ps3d_objx_close(h);
        return rc;
    }
    if (m.num_indices) {
        ps3d_objx_close(h);
        return report_error(PS3D_ERR_INVALID, "indexed OBJX meshes are not drawable as vertex arrays");
    }
    if (m.has_texcoords && !m.has_normals) {
        ps3d_objx_close(h);
        return report_error(PS3D_ERR_INVALID, "binormals need normals");
    }
    const size_t nv = m.num_vertices;
    std::vector<float> pos(4 * nv), nrm(m.has_normals ? 4 * nv : 0), tan(m.has_texcoords ? 4 * nv : 0),
        uv(m.has_texcoords ? 2 * nv : 0), bin(m.has_texcoords ? 4 * nv : 0);
    rc = ps3d_objx_read_mesh(h, pos.data(), m.has_normals ? nrm.data() : nullptr,
                             m.has_texcoords ? tan.data() : nullptr, m.has_texcoords ? uv.data() : nullptr, nullptr);
    ps3d_objx_close(h);
    if (rc) return rc;
    // scenobj.cpp:117-131: positions get w = 1; binormal = norm(cross(n, t))
    for (size_t i = 0; i < nv; i++) pos[4 * i + 3] = 1.0f;
    if (m.has_texcoords)
        for (size_t i = 0; i < nv; i++) {
            cross3(&bin[4 * i], &nrm[4 * i], &tan[4 * i]);
            norm4(&bin[4 * i]);
        }
    int vao = ps3d_vao_create(p);
    if (vao < 0) return vao;
    const int n = (int)nv;
    if ((rc = ps3d_vbo_attach(p, vao, 0, 16, n, pos.data())) < 0) return rc;
    if (m.has_texcoords) {
        if ((rc = ps3d_vbo_attach(p, vao, 1, 16, n, tan.data())) < 0) return rc;
        if ((rc = ps3d_vbo_attach(p, vao, 2, 16, n, bin.data())) < 0) return rc;
        if ((rc = ps3d_vbo_attach(p, vao, 4, 8, n, uv.data())) < 0) return rc;
    }
    if (m.has_normals && (rc = ps3d_vbo_attach(p, vao, 3, 16, n, nrm.data())) < 0) return rc;
    *vaoOut = vao;
    return 0;
}

}  // extern "C"
