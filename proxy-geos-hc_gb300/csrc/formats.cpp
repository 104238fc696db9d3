// formats.cpp -- on-disk formats of the solver's outputs (sem_traces_*, sem_snapshot_*).
//
// One container for both: 8-byte magic, little-endian uint64 header length, a UTF-8 JSON header,
// zero padding to a 64-byte boundary, then little-endian float32 samples.
//   traces    magic "SEMTRC01": trace-major samples [n_traces][n_samples] (SEG-Y's order: one
//             receiver's whole time series after another), header with dt, receiver and source
//             coordinates and free-form caller metadata;
//   snapshot  magic "SEMSNP01": one x-z plane of a pressure level [nz][nx] (row = fixed z), header
//             with the plane index, step, level and the node coordinates along x and z.  The
//             reference writes this plane as ASCII "x z value" lines (SEMmesh.cpp:624-654, plane
//             y = ny/2 - 1); the binary container replaces it.
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "abi.h"
#include "solver.h"

using namespace semgb;

namespace {

constexpr char kTraceMagic[9] = "SEMTRC01";
constexpr char kSnapMagic[9] = "SEMSNP01";

void put_u64(unsigned char *p, uint64_t v)
{
    for (int i = 0; i < 8; i++) p[i] = (unsigned char)(v >> (8 * i));
}

uint64_t get_u64(const unsigned char *p)
{
    uint64_t v = 0;
    for (int i = 0; i < 8; i++) v |= (uint64_t)p[i] << (8 * i);
    return v;
}

std::string num(double v)
{
    if (!std::isfinite(v)) return "null";
    char b[40];
    std::snprintf(b, sizeof b, "%.9g", v);
    return b;
}

std::string xyz_list(int n, const float *xyz)
{
    std::string s = "[";
    for (int i = 0; i < n; i++) {
        if (i) s += ",";
        s += "[" + num(xyz[3 * i]) + "," + num(xyz[3 * i + 1]) + "," + num(xyz[3 * i + 2]) + "]";
    }
    return s + "]";
}

std::string num_list(int n, const double *v)
{
    std::string s = "[";
    for (int i = 0; i < n; i++) s += (i ? "," : "") + num(v[i]);
    return s + "]";
}

// float32 samples in little-endian byte order whatever the host's
void put_f32(std::vector<unsigned char> &out, float v)
{
    uint32_t u;
    std::memcpy(&u, &v, 4);
    for (int i = 0; i < 4; i++) out.push_back((unsigned char)(u >> (8 * i)));
}

int write_container(const char *path, const char *magic, const std::string &json, const std::vector<unsigned char> &data)
{
    std::FILE *f = std::fopen(path, "wb");
    if (!f) return sem_fail(SEM_ERR_ARG, std::string("cannot open ") + path + " for writing");
    unsigned char head[16];
    std::memcpy(head, magic, 8);
    put_u64(head + 8, json.size());
    const size_t used = 16 + json.size();
    const size_t pad = (64 - used % 64) % 64;
    const std::vector<unsigned char> zeros(pad, 0);
    bool ok = std::fwrite(head, 1, 16, f) == 16 && std::fwrite(json.data(), 1, json.size(), f) == json.size() &&
              std::fwrite(zeros.data(), 1, pad, f) == pad &&
              std::fwrite(data.data(), 1, data.size(), f) == data.size();
    ok = std::fclose(f) == 0 && ok;
    return ok ? SEM_OK : sem_fail(SEM_ERR_ARG, std::string("write failed: ") + path);
}

// Reads the header (JSON text) and the data offset; returns SEM_OK or an error.
int read_container(const char *path, const char *magic, std::string &json, uint64_t &data_off, uint64_t &file_size)
{
    std::FILE *f = std::fopen(path, "rb");
    if (!f) return sem_fail(SEM_ERR_ARG, std::string("cannot open ") + path);
    unsigned char head[16];
    if (std::fread(head, 1, 16, f) != 16 || std::memcmp(head, magic, 8) != 0) {
        std::fclose(f);
        return sem_fail(SEM_ERR_ARG, std::string(path) + ": not a " + magic + " file");
    }
    const uint64_t n = get_u64(head + 8);
    if (n > (1u << 30)) {
        std::fclose(f);
        return sem_fail(SEM_ERR_ARG, std::string(path) + ": header too large");
    }
    json.assign(n, '\0');
    const bool ok = std::fread(&json[0], 1, n, f) == n;
    std::fseek(f, 0, SEEK_END);
    file_size = (uint64_t)std::ftell(f);
    std::fclose(f);
    if (!ok) return sem_fail(SEM_ERR_ARG, std::string(path) + ": truncated header");
    data_off = (16 + n + 63) / 64 * 64;
    return SEM_OK;
}

// Minimal reader of one integer or number field of the writer's own JSON ("key": value).
bool json_number(const std::string &j, const char *key, double &v)
{
    const std::string k = std::string("\"") + key + "\":";
    const size_t p = j.find(k);
    if (p == std::string::npos) return false;
    char *end = nullptr;
    v = std::strtod(j.c_str() + p + k.size(), &end);
    return end != j.c_str() + p + k.size();
}

int read_f32(const char *path, uint64_t off, size_t n, float *out)
{
    std::FILE *f = std::fopen(path, "rb");
    if (!f) return sem_fail(SEM_ERR_ARG, std::string("cannot open ") + path);
    std::vector<unsigned char> b(n * 4);
    const bool ok = std::fseek(f, (long)off, SEEK_SET) == 0 && std::fread(b.data(), 1, b.size(), f) == b.size();
    std::fclose(f);
    if (!ok) return sem_fail(SEM_ERR_ARG, std::string(path) + ": truncated data");
    for (size_t i = 0; i < n; i++) {
        const uint32_t u = (uint32_t)b[4 * i] | (uint32_t)b[4 * i + 1] << 8 | (uint32_t)b[4 * i + 2] << 16 |
                           (uint32_t)b[4 * i + 3] << 24;
        std::memcpy(out + i, &u, 4);
    }
    return SEM_OK;
}

}  // namespace

extern "C" {

int sem_traces_write(const char *path, int n_steps, int n_rec, const float *traces, float dt, const float *rec_xyz,
                     int n_src, const float *src_xyz, const char *extra_json)
{
    GUARD_BEGIN
    if (!path || n_steps < 0 || n_rec < 0 || n_src < 0 || (n_steps * (int64_t)n_rec > 0 && !traces) ||
        (n_src > 0 && !src_xyz))
        return sem_fail(SEM_ERR_ARG, "bad arguments");
    std::string j = "{\"format\":\"semgb-traces\",\"version\":1,\"n_traces\":" + std::to_string(n_rec) +
                    ",\"n_samples\":" + std::to_string(n_steps) + ",\"dt\":" + num(dt) +
                    ",\"sample_format\":\"float32-le\",\"order\":\"trace-major\",\"receivers\":" +
                    (rec_xyz ? xyz_list(n_rec, rec_xyz) : std::string("null")) + ",\"sources\":" +
                    xyz_list(n_src, src_xyz) + ",\"extra\":" + (extra_json && *extra_json ? extra_json : "null") + "}";
    std::vector<unsigned char> data;
    data.reserve((size_t)n_steps * n_rec * 4);
    for (int r = 0; r < n_rec; r++)
        for (int t = 0; t < n_steps; t++) put_f32(data, traces[(size_t)t * n_rec + r]);
    return write_container(path, kTraceMagic, j, data);
    GUARD_END
}

int sem_traces_read_info(const char *path, int *n_steps, int *n_rec, float *dt)
{
    GUARD_BEGIN
    std::string j;
    uint64_t off = 0, size = 0;
    int rc = read_container(path, kTraceMagic, j, off, size);
    if (rc) return rc;
    double ns = 0, nr = 0, d = 0;
    if (!json_number(j, "n_samples", ns) || !json_number(j, "n_traces", nr) || !json_number(j, "dt", d))
        return sem_fail(SEM_ERR_ARG, std::string(path) + ": header lacks n_samples, n_traces or dt");
    if (size < off + (uint64_t)(ns * nr * 4)) return sem_fail(SEM_ERR_ARG, std::string(path) + ": truncated data");
    if (n_steps) *n_steps = (int)ns;
    if (n_rec) *n_rec = (int)nr;
    if (dt) *dt = (float)d;
    return SEM_OK;
    GUARD_END
}

int sem_traces_read(const char *path, float *traces)
{
    GUARD_BEGIN
    int ns = 0, nr = 0;
    int rc = sem_traces_read_info(path, &ns, &nr, nullptr);
    if (rc) return rc;
    if (!traces) return sem_fail(SEM_ERR_ARG, "NULL output");
    std::string j;
    uint64_t off = 0, size = 0;
    if ((rc = read_container(path, kTraceMagic, j, off, size))) return rc;
    std::vector<float> tm((size_t)ns * nr);
    if ((rc = read_f32(path, off, tm.size(), tm.data()))) return rc;
    for (int r = 0; r < nr; r++)
        for (int t = 0; t < ns; t++) traces[(size_t)t * nr + r] = tm[(size_t)r * ns + t];
    return SEM_OK;
    GUARD_END
}

int sem_solver_write_snapshot(sem_solver *s, int level, int y_index, const char *path)
{
    GUARD_BEGIN
    if (!s || !path) return sem_fail(SEM_ERR_ARG, "NULL argument");
    const Box &b = s->mesh->box;
    if (y_index < 0) y_index = b.ny == 1 ? 0 : (int)(b.ny / 2 - 1);  // the reference's plane
    if (y_index >= b.ny) return sem_fail(SEM_ERR_ARG, "plane index out of range");
    std::vector<float> p((size_t)b.n_nodes);
    int rc = sem_solver_get_pressure(s, level, p.data());
    if (rc) return rc;
    // node coordinates along x and z (GLL points inside each element)
    auto axis = [&](int ne, double len, std::vector<double> &c) {
        const int n = ne * b.order + 1;
        c.resize(n);
        const double h = len / ne;
        for (int i = 0; i < n; i++) {
            int e = i / b.order, l = i - e * b.order;
            if (e == ne) { e = ne - 1; l = b.order; }
            c[i] = e * h + (1.0 + s->mesh->gll.xi[l]) * 0.5 * h;
        }
    };
    std::vector<double> cx, cz;
    axis(b.ex, b.lx, cx);
    axis(b.ez, b.lz, cz);
    const std::string j = "{\"format\":\"semgb-snapshot\",\"version\":1,\"nx\":" + std::to_string(b.nx) +
                          ",\"nz\":" + std::to_string(b.nz) + ",\"y_index\":" + std::to_string(y_index) +
                          ",\"step\":" + std::to_string(s->steps_done) + ",\"level\":\"" +
                          (level == SEM_LEVEL_PREVIOUS ? "previous" : "current") +
                          "\",\"sample_format\":\"float32-le\",\"order\":\"z-major rows of x\",\"x\":" +
                          num_list((int)cx.size(), cx.data()) + ",\"z\":" + num_list((int)cz.size(), cz.data()) + "}";
    std::vector<unsigned char> data;
    data.reserve((size_t)b.nx * b.nz * 4);
    const size_t base = (size_t)y_index * b.nx * b.nz;
    for (int64_t i = 0; i < b.nx * b.nz; i++) put_f32(data, p[base + i]);
    return write_container(path, kSnapMagic, j, data);
    GUARD_END
}

int sem_snapshot_read_info(const char *path, int *nx, int *nz, int *y_index)
{
    GUARD_BEGIN
    std::string j;
    uint64_t off = 0, size = 0;
    int rc = read_container(path, kSnapMagic, j, off, size);
    if (rc) return rc;
    double x = 0, z = 0, y = 0;
    if (!json_number(j, "nx", x) || !json_number(j, "nz", z) || !json_number(j, "y_index", y))
        return sem_fail(SEM_ERR_ARG, std::string(path) + ": header lacks nx, nz or y_index");
    if (size < off + (uint64_t)(x * z * 4)) return sem_fail(SEM_ERR_ARG, std::string(path) + ": truncated data");
    if (nx) *nx = (int)x;
    if (nz) *nz = (int)z;
    if (y_index) *y_index = (int)y;
    return SEM_OK;
    GUARD_END
}

int sem_snapshot_read(const char *path, float *plane)
{
    GUARD_BEGIN
    int nx = 0, nz = 0;
    int rc = sem_snapshot_read_info(path, &nx, &nz, nullptr);
    if (rc) return rc;
    if (!plane) return sem_fail(SEM_ERR_ARG, "NULL output");
    std::string j;
    uint64_t off = 0, size = 0;
    if ((rc = read_container(path, kSnapMagic, j, off, size))) return rc;
    return read_f32(path, off, (size_t)nx * nz, plane);
    GUARD_END
}

}  // extern "C"
