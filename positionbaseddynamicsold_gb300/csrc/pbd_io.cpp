// pbd_io.cpp -- the reference's text caches and text scene files, on the host.
//
// Cache format (Buffer::Save, P/Buffer.cuh:70-80; IO::SaveData,
// P/PBD_Basic.cuh:262-278): one line per buffer, `name|type|v;v;...;`, values
// printed by a default-formatted output stream (6 significant digits),
// float3 as `x,y,z` and int2 as `x,y` (P/PBD_Basic.cuh:69-79); scalars as
// `name|type|value`.  The readers (IO::ReadTopolFromCache / Read-
// ConstraintFromCache, P/PBD_Basic.cuh:326-530) split a line at '|', skip it
// unless it has exactly three fields, split the third at ';' and convert with
// stoi / stof; the type field is not read.  A topology cache carries
// Indices, P, primList (triangles), velBuffer, massBuffer, dampingRate,
// gravity (PBDObject::SaveMeshTopol, P/PBD_cuda.cu:907-925); a constraint
// cache carries Indices, P, primList, prdPBuffer, restPosBuffer,
// restLengthBuffer, stiffnessBuffer, constraintType (ConstraintPBD::Save,
// P/PBD_cuda.cu:627-640).  PBDObject::ContinueSimInit (P/PBD_cuda.cu:660-667)
// is the two readers in a row.
//
// Text scene files (IO::ReadTopolFromTxt / ReadDistConstrFromTxt,
// P/PBD_Basic.cuh:532-660): the topology file's first line holds `label:`
// then x,y,z,... and its second line `label:` then triangle corner ids; each
// point gets massBuffer 1 and zero velocity.  The constraint file's first
// line is skipped; each further line holds `label:` then pairs i0,i1 of
// distance constraints, with the given stiffness and the rest length of the
// positions spelled as the reference's IO::Distance (powf).
//
// Differences from the reference (each documented in the header):
//  - a line ending in '\r' (a file written on Windows, read here) has it
//    removed first;
//  - a field that does not convert is an error (PBD_ERR_ARG with the line
//    number) where stoi / stof would throw;
//  - distance constraints of a second data line of the text constraint file
//    start after those of the first (the reference restarts their primList
//    offsets at 0 on every line, pointing them at the wrong indices);
//  - the type field written is the reference's Windows spelling (`int`,
//    `float`, `struct float3`, `struct int2`); it is not read back.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "pbd_common.cuh"

struct pbd_scene {
    std::vector<float> pos, vel, mass;   // 3n, 3n, n
    std::vector<int> tri;                // 3 per triangle
    std::vector<int> prim_list, indices, ctype;
    std::vector<float> rest_length, stiffness;
    std::vector<float> prdp;             // constraint cache prdPBuffer (3n or empty)
    float damping = 1.0f;
    float gravity[3] = {0.f, 0.f, 0.f};
    int has_damping = 0, has_gravity = 0;
    pbd_object_desc desc;
};

namespace {

using pbd::set_error;

std::vector<std::string> split(const std::string &src, const std::string &sep) {
    // UT::splitString (P/Utility.h:8-28): pieces between separators; a
    // trailing separator yields no empty last piece
    std::vector<std::string> v;
    std::string::size_type p1 = 0, p2 = src.find(sep);
    while (p2 != std::string::npos) {
        v.push_back(src.substr(p1, p2 - p1));
        p1 = p2 + sep.size();
        p2 = src.find(sep, p1);
    }
    if (p1 != src.length()) v.push_back(src.substr(p1));
    return v;
}

bool to_int(const std::string &s, int &out) {
    const char *b = s.c_str();
    char *e = nullptr;
    long v = strtol(b, &e, 10);
    if (e == b) return false;
    out = (int)v;
    return true;
}
bool to_float(const std::string &s, float &out) {
    const char *b = s.c_str();
    char *e = nullptr;
    float v = strtof(b, &e);
    if (e == b) return false;
    out = v;
    return true;
}

struct LineReader {
    std::ifstream in;
    std::string path;
    int line = 0;
    explicit LineReader(const char *p) : in(p), path(p) {}
    bool next(std::string &s) {
        if (!std::getline(in, s)) return false;
        ++line;
        if (!s.empty() && s.back() == '\r') s.pop_back();
        return true;
    }
};

#define IO_FAIL(rd, what)                                                                    \
    do {                                                                                     \
        set_error("%s:%d: %s", (rd).path.c_str(), (rd).line, what);                          \
        return PBD_ERR_ARG;                                                                  \
    } while (0)

int parse_ints(LineReader &rd, const std::vector<std::string> &items, std::vector<int> &out) {
    for (const auto &it : items) {
        int v;
        if (!to_int(it, v)) IO_FAIL(rd, "not an integer");
        out.push_back(v);
    }
    return PBD_OK;
}
int parse_floats(LineReader &rd, const std::vector<std::string> &items, std::vector<float> &out) {
    for (const auto &it : items) {
        float v;
        if (!to_float(it, v)) IO_FAIL(rd, "not a number");
        out.push_back(v);
    }
    return PBD_OK;
}
// tuples `a,b[,c]` separated by ';'
int parse_tuples_f(LineReader &rd, const std::vector<std::string> &items, int k,
                   std::vector<float> &out) {
    for (const auto &it : items) {
        auto parts = split(it, ",");
        if ((int)parts.size() < k) IO_FAIL(rd, "short tuple");
        for (int j = 0; j < k; ++j) {
            float v;
            if (!to_float(parts[j], v)) IO_FAIL(rd, "not a number");
            out.push_back(v);
        }
    }
    return PBD_OK;
}
int parse_tuples_i(LineReader &rd, const std::vector<std::string> &items, int k,
                   std::vector<int> &out) {
    for (const auto &it : items) {
        auto parts = split(it, ",");
        if ((int)parts.size() < k) IO_FAIL(rd, "short tuple");
        for (int j = 0; j < k; ++j) {
            int v;
            if (!to_int(parts[j], v)) IO_FAIL(rd, "not an integer");
            out.push_back(v);
        }
    }
    return PBD_OK;
}

void fill_desc(pbd_scene *s) {
    pbd_object_desc &d = s->desc;
    memset(&d, 0, sizeof(d));
    d.n_points = (int)s->mass.size();
    d.pos = s->pos.data();
    d.vel = s->vel.size() == s->pos.size() ? s->vel.data() : nullptr;
    d.mass = s->mass.data();
    d.n_tris = (int)s->tri.size() / 3;
    d.tri_idx = d.n_tris ? s->tri.data() : nullptr;
    d.n_prims = (int)s->ctype.size();
    if (d.n_prims) {
        d.prim_list = s->prim_list.data();
        d.indices = s->indices.data();
        d.constraint_type = s->ctype.data();
        d.rest_length = s->rest_length.data();
        d.stiffness = s->stiffness.data();
    }
    d.damping_rate = s->damping;
    for (int k = 0; k < 3; ++k) d.gravity[k] = s->gravity[k];
}

// IO::ReadTopolFromCache (P/PBD_Basic.cuh:326-425)
int read_topol_cache(const char *path, pbd_scene *s) {
    LineReader rd(path);
    PBD_CHECK(rd.in.is_open(), PBD_ERR_ARG, "cannot open %s", path);
    std::vector<int> idx, prims;
    std::string line;
    while (rd.next(line)) {
        auto f = split(line, "|");
        if (f.size() != 3) continue;
        auto items = split(f[2], ";");
        const std::string &name = f[0];
        if (name == "Indices") PBD_TRY(parse_ints(rd, items, idx));
        else if (name == "P") PBD_TRY(parse_tuples_f(rd, items, 3, s->pos));
        else if (name == "primList") PBD_TRY(parse_tuples_i(rd, items, 2, prims));
        else if (name == "velBuffer") PBD_TRY(parse_tuples_f(rd, items, 3, s->vel));
        else if (name == "massBuffer") PBD_TRY(parse_floats(rd, items, s->mass));
        else if (name == "dampingRate") {
            std::vector<float> v;
            PBD_TRY(parse_floats(rd, items, v));
            if (v.empty()) IO_FAIL(rd, "dampingRate without a value");
            s->damping = v[0];
            s->has_damping = 1;
        } else if (name == "gravity") {
            std::vector<float> v;
            if (items.empty()) IO_FAIL(rd, "gravity without a value");
            PBD_TRY(parse_tuples_f(rd, {items[0]}, 3, v));
            for (int k = 0; k < 3; ++k) s->gravity[k] = v[k];
            s->has_gravity = 1;
        }
    }
    // triangles: the mesh primList holds (start, 3) ranges of Indices
    for (size_t p = 0; p + 1 < prims.size(); p += 2) {
        int st = prims[p], cnt = prims[p + 1];
        PBD_CHECK(cnt == 3, PBD_ERR_ARG, "%s: mesh prim %zu has %d points (triangles only)",
                  path, p / 2, cnt);
        PBD_CHECK(st >= 0 && st + 3 <= (int)idx.size(), PBD_ERR_ARG,
                  "%s: mesh prim %zu outside Indices", path, p / 2);
        for (int k = 0; k < 3; ++k) s->tri.push_back(idx[st + k]);
    }
    const size_t n = s->pos.size() / 3;
    if (s->mass.empty()) s->mass.assign(n, 1.0f);
    PBD_CHECK(s->mass.size() == n, PBD_ERR_ARG, "%s: %zu massBuffer values for %zu points", path,
              s->mass.size(), n);
    PBD_CHECK(s->vel.empty() || s->vel.size() == 3 * n, PBD_ERR_ARG,
              "%s: velBuffer does not match P", path);
    return PBD_OK;
}

// IO::ReadConstraintFromCache (P/PBD_Basic.cuh:427-530)
int read_constr_cache(const char *path, pbd_scene *s) {
    LineReader rd(path);
    PBD_CHECK(rd.in.is_open(), PBD_ERR_ARG, "cannot open %s", path);
    std::vector<float> cpos;
    std::string line;
    while (rd.next(line)) {
        auto f = split(line, "|");
        if (f.size() != 3) continue;
        auto items = split(f[2], ";");
        const std::string &name = f[0];
        if (name == "Indices") PBD_TRY(parse_ints(rd, items, s->indices));
        else if (name == "P") PBD_TRY(parse_tuples_f(rd, items, 3, cpos));
        else if (name == "primList") PBD_TRY(parse_tuples_i(rd, items, 2, s->prim_list));
        // the reference appends both prdPBuffer and restPosBuffer lines to the
        // predicted positions (P/PBD_Basic.cuh:494-511)
        else if (name == "prdPBuffer" || name == "restPosBuffer")
            PBD_TRY(parse_tuples_f(rd, items, 3, s->prdp));
        else if (name == "restLengthBuffer") PBD_TRY(parse_floats(rd, items, s->rest_length));
        else if (name == "stiffnessBuffer") PBD_TRY(parse_floats(rd, items, s->stiffness));
        else if (name == "constraintType") PBD_TRY(parse_ints(rd, items, s->ctype));
    }
    const size_t np = s->prim_list.size() / 2;
    PBD_CHECK(s->ctype.size() == np && s->stiffness.size() == np, PBD_ERR_ARG,
              "%s: %zu prims, %zu types, %zu stiffnesses", path, np, s->ctype.size(),
              s->stiffness.size());
    if (s->rest_length.size() < np) s->rest_length.resize(np, 0.f);
    if (s->pos.empty()) s->pos = cpos;   // a constraint cache read on its own
    return PBD_OK;
}

float ref_distance(const float *a, const float *b) {
    // IO::Distance (P/PBD_Basic.cuh:321-324)
    return powf(powf(a[0] - b[0], 2) + powf(a[1] - b[1], 2) + powf(a[2] - b[2], 2), 0.5f);
}

// IO::ReadTopolFromTxt (P/PBD_Basic.cuh:532-600)
int read_topol_txt(const char *path, pbd_scene *s) {
    LineReader rd(path);
    PBD_CHECK(rd.in.is_open(), PBD_ERR_ARG, "cannot open %s", path);
    std::string line;
    int k = 0;
    while (rd.next(line)) {
        auto f = split(line, ":");
        if (f.size() < 2) IO_FAIL(rd, "no ':' in the line");
        auto items = split(f[1], ",");
        if (k == 0) {
            PBD_TRY(parse_floats(rd, items, s->pos));
            if (s->pos.size() % 3) IO_FAIL(rd, "positions are not triples");
        } else {
            std::vector<int> ids;
            PBD_TRY(parse_ints(rd, items, ids));
            if (ids.size() % 3) IO_FAIL(rd, "triangle corners are not triples");
            s->tri.insert(s->tri.end(), ids.begin(), ids.end());
        }
        ++k;
    }
    const size_t n = s->pos.size() / 3;
    s->mass.assign(n, 1.0f);
    s->vel.assign(3 * n, 0.0f);
    return PBD_OK;
}

// IO::ReadDistConstrFromTxt (P/PBD_Basic.cuh:602-660)
int read_dist_txt(const char *path, float stiffness, pbd_scene *s) {
    LineReader rd(path);
    PBD_CHECK(rd.in.is_open(), PBD_ERR_ARG, "cannot open %s", path);
    const int n = (int)(s->pos.size() / 3);
    std::string line;
    int k = 0;
    while (rd.next(line)) {
        if (k++ == 0) continue;  // the first line is not used
        auto f = split(line, ":");
        if (f.size() < 2) IO_FAIL(rd, "no ':' in the line");
        std::vector<int> ids;
        PBD_TRY(parse_ints(rd, split(f[1], ","), ids));
        if (ids.size() % 2) IO_FAIL(rd, "constraint ends are not pairs");
        for (size_t i = 0; i < ids.size(); i += 2) {
            int a = ids[i], b = ids[i + 1];
            if (a < 0 || a >= n || b < 0 || b >= n) IO_FAIL(rd, "point id out of range");
            s->prim_list.push_back((int)s->indices.size());
            s->prim_list.push_back(2);
            s->indices.push_back(a);
            s->indices.push_back(b);
            s->ctype.push_back(PBD_DISTANCE);
            s->stiffness.push_back(stiffness);
            s->rest_length.push_back(ref_distance(&s->pos[3 * a], &s->pos[3 * b]));
        }
    }
    return PBD_OK;
}

// output stream formatting of the reference's writers
struct Out {
    std::ostringstream os;
    void f(float v) { os << v; }
    void i(int v) { os << v; }
};

void write_line_i(Out &o, const char *name, const int *v, size_t n) {
    o.os << name << "|int|";
    for (size_t k = 0; k < n; ++k) {
        o.i(v[k]);
        o.os << ";";
    }
    o.os << "\n";
}
void write_line_f(Out &o, const char *name, const float *v, size_t n) {
    o.os << name << "|float|";
    for (size_t k = 0; k < n; ++k) {
        o.f(v[k]);
        o.os << ";";
    }
    o.os << "\n";
}
void write_line_f3(Out &o, const char *name, const float *v, size_t n) {
    o.os << name << "|struct float3|";
    for (size_t k = 0; k < n; ++k) {
        o.f(v[3 * k]);
        o.os << ",";
        o.f(v[3 * k + 1]);
        o.os << ",";
        o.f(v[3 * k + 2]);
        o.os << ";";
    }
    o.os << "\n";
}
void write_line_i2(Out &o, const char *name, const int *v, size_t n) {
    o.os << name << "|struct int2|";
    for (size_t k = 0; k < n; ++k) {
        o.i(v[2 * k]);
        o.os << ",";
        o.i(v[2 * k + 1]);
        o.os << ";";
    }
    o.os << "\n";
}

int write_file(const char *path, const std::string &text) {
    std::ofstream ofs(path, std::ios::binary);
    PBD_CHECK(ofs.is_open(), PBD_ERR_ARG, "cannot write %s", path);
    ofs << text;
    ofs.close();
    PBD_CHECK(!ofs.fail(), PBD_ERR_ARG, "writing %s failed", path);
    return PBD_OK;
}

}  // namespace

extern "C" {

int pbd_scene_read_cache(const char *topol_path, const char *constr_path, pbd_scene **out) {
    PBD_CHECK(out && (topol_path || constr_path), PBD_ERR_ARG, "null argument");
    *out = nullptr;
    pbd_scene *s = new pbd_scene();
    int r = PBD_OK;
    if (topol_path) r = read_topol_cache(topol_path, s);
    if (r == PBD_OK && constr_path) r = read_constr_cache(constr_path, s);
    if (r != PBD_OK) {
        delete s;
        return r;
    }
    if (s->mass.size() != s->pos.size() / 3) s->mass.assign(s->pos.size() / 3, 1.0f);
    fill_desc(s);
    *out = s;
    return PBD_OK;
}

int pbd_scene_read_txt(const char *topol_path, const char *dist_constr_path, float stiffness,
                       pbd_scene **out) {
    PBD_CHECK(out && topol_path, PBD_ERR_ARG, "null argument");
    *out = nullptr;
    pbd_scene *s = new pbd_scene();
    int r = read_topol_txt(topol_path, s);
    if (r == PBD_OK && dist_constr_path) r = read_dist_txt(dist_constr_path, stiffness, s);
    if (r != PBD_OK) {
        delete s;
        return r;
    }
    fill_desc(s);
    *out = s;
    return PBD_OK;
}

int pbd_scene_desc(pbd_scene *s, pbd_object_desc *desc, const float **predicted,
                   int *has_damping, int *has_gravity) {
    PBD_CHECK(s && desc, PBD_ERR_ARG, "null argument");
    *desc = s->desc;
    if (predicted)
        *predicted = s->prdp.size() == s->pos.size() && !s->prdp.empty() ? s->prdp.data() : nullptr;
    if (has_damping) *has_damping = s->has_damping;
    if (has_gravity) *has_gravity = s->has_gravity;
    return PBD_OK;
}

int pbd_scene_destroy(pbd_scene *s) {
    delete s;
    return PBD_OK;
}

int pbd_scene_write_cache(const pbd_object_desc *d, const float *predicted,
                          const char *topol_path, const char *constr_path) {
    PBD_CHECK(d && d->pos && d->mass && d->n_points > 0, PBD_ERR_ARG, "bad scene");
    const size_t n = (size_t)d->n_points;
    if (topol_path) {
        // PBDObject::SaveMeshTopol (P/PBD_cuda.cu:907-925)
        Out o;
        std::vector<int> idx(3 * (size_t)d->n_tris), prims(2 * (size_t)d->n_tris);
        for (int t = 0; t < d->n_tris; ++t) {
            for (int k = 0; k < 3; ++k) idx[3 * t + k] = d->tri_idx[3 * t + k];
            prims[2 * t] = 3 * t;
            prims[2 * t + 1] = 3;
        }
        std::vector<float> zero;
        const float *vel = d->vel;
        if (!vel) {
            zero.assign(3 * n, 0.f);
            vel = zero.data();
        }
        write_line_i(o, "Indices", idx.data(), idx.size());
        write_line_f3(o, "P", d->pos, n);
        write_line_i2(o, "primList", prims.data(), (size_t)d->n_tris);
        write_line_f3(o, "velBuffer", vel, n);
        write_line_f(o, "massBuffer", d->mass, n);
        o.os << "dampingRate|float|";
        o.f(d->damping_rate);
        o.os << "\n";
        o.os << "gravity|struct float3|";
        o.f(d->gravity[0]);
        o.os << ",";
        o.f(d->gravity[1]);
        o.os << ",";
        o.f(d->gravity[2]);
        o.os << "\n";
        PBD_TRY(write_file(topol_path, o.os.str()));
    }
    if (constr_path) {
        // PBDObject::SaveConstraint / ConstraintPBD::Save (P/PBD_cuda.cu:627-640, 927-938)
        PBD_CHECK(d->n_prims == 0 || (d->prim_list && d->indices && d->constraint_type &&
                                      d->stiffness),
                  PBD_ERR_ARG, "bad constraint buffers");
        int n_idx = 0;
        for (int p = 0; p < d->n_prims; ++p)
            n_idx = std::max(n_idx, d->prim_list[2 * p] + d->prim_list[2 * p + 1]);
        std::vector<float> rl((size_t)d->n_prims, 0.f);
        if (d->rest_length)
            for (int p = 0; p < d->n_prims; ++p) rl[p] = d->rest_length[p];
        Out o;
        write_line_i(o, "Indices", d->indices, (size_t)n_idx);
        write_line_f3(o, "P", d->pos, n);
        write_line_i2(o, "primList", d->prim_list, (size_t)d->n_prims);
        write_line_f3(o, "prdPBuffer", predicted ? predicted : d->pos, n);
        write_line_f3(o, "restPosBuffer", nullptr, 0);
        write_line_f(o, "restLengthBuffer", rl.data(), rl.size());
        write_line_f(o, "stiffnessBuffer", d->stiffness, (size_t)d->n_prims);
        write_line_i(o, "constraintType", d->constraint_type, (size_t)d->n_prims);
        PBD_TRY(write_file(constr_path, o.os.str()));
    }
    return PBD_OK;
}

}  // extern "C"

extern "C" {

int pbd_object_create_from_cache(const char *topol_path, const char *constr_path,
                                 pbd_object **out) {
    PBD_CHECK(out && topol_path && constr_path, PBD_ERR_ARG, "null argument");
    pbd_scene *s = nullptr;
    PBD_TRY(pbd_scene_read_cache(topol_path, constr_path, &s));
    int r = pbd_object_create(&s->desc, out);
    if (r == PBD_OK && s->prdp.size() == s->pos.size() && !s->prdp.empty()) {
        r = pbd_object_set_predicted(*out, s->prdp.data());
        if (r != PBD_OK) {
            pbd_object_destroy(*out);
            *out = nullptr;
        }
    }
    pbd_scene_destroy(s);
    return r;
}

int pbd_object_save_cache(pbd_object *o, const char *topol_path, const char *constr_path) {
    PBD_CHECK(o && (topol_path || constr_path), PBD_ERR_ARG, "null argument");
    const int n = o->n;
    std::vector<float> pos(3 * (size_t)n), vel(3 * (size_t)n), prd(3 * (size_t)n);
    PBD_TRY(pbd_object_get_positions(o, pos.data()));
    PBD_TRY(pbd_object_get_velocities(o, vel.data()));
    PBD_TRY(pbd_object_get_predicted(o, prd.data()));
    std::vector<int4> tri4((size_t)o->nt);
    std::vector<int> tri(3 * (size_t)o->nt);
    std::vector<float> stiff((size_t)o->np);
    if (o->nt)
        PBD_CUDA(cudaMemcpyAsync(tri4.data(), o->tri.p, sizeof(int4) * o->nt,
                                 cudaMemcpyDeviceToHost, o->stream));
    if (o->np)
        PBD_CUDA(cudaMemcpyAsync(stiff.data(), o->stiffness.p, sizeof(float) * o->np,
                                 cudaMemcpyDeviceToHost, o->stream));
    PBD_CUDA(cudaStreamSynchronize(o->stream));
    for (int t = 0; t < o->nt; ++t) {
        tri[3 * t] = tri4[t].x;
        tri[3 * t + 1] = tri4[t].y;
        tri[3 * t + 2] = tri4[t].z;
    }
    pbd_object_desc d;
    memset(&d, 0, sizeof(d));
    d.n_points = n;
    d.pos = pos.data();
    d.vel = vel.data();
    d.mass = o->h_mass.data();
    d.n_tris = o->nt;
    d.tri_idx = tri.data();
    d.n_prims = o->np;
    d.prim_list = o->h_prim_list.data();
    d.indices = o->h_indices.data();
    d.constraint_type = o->h_ctype.data();
    d.rest_length = o->h_rest_length.data();
    d.stiffness = stiff.data();
    d.damping_rate = o->damping;
    for (int k = 0; k < 3; ++k) d.gravity[k] = o->gravity[k];
    return pbd_scene_write_cache(&d, prd.data(), topol_path, constr_path);
}

}  // extern "C"
