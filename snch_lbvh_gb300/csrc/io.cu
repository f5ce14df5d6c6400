// Host-side file formats of libsnch_gb300: Wavefront OBJ meshes
// (scene_loader<3>, include/snch_lbvh/scene_loader.cuh:86-152).
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "internal.h"

namespace
{

// next whitespace-separated token of s starting at *pos (empty at the end)
std::string token(const std::string &s, size_t *pos)
{
    size_t i = *pos;
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\r' || s[i] == '\f' || s[i] == '\v'))
        ++i;
    size_t j = i;
    while (j < s.size() && !(s[j] == ' ' || s[j] == '\t' || s[j] == '\r' || s[j] == '\f' || s[j] == '\v'))
        ++j;
    *pos = j;
    return s.substr(i, j - i);
}

// istream >> float / int as the reference reads them: a failed or missing
// number gives 0 (C++11 extraction failure), and so does every later field of
// the line (the reference leaves those unset: its stream stays failed)
struct Fields
{
    bool failed = false;
    float f(const std::string &t)
    {
        if (failed || t.empty())
            return failed = true, 0.0f;
        char *end = nullptr;
        errno = 0;
        const float v = std::strtof(t.c_str(), &end);
        if (end == t.c_str())
            return failed = true, 0.0f;
        return v;
    }
    // the vertex index of a face token: "7", or the "7" of "7/1/3", "7//3".
    // (The reference's stream reads the 7 of "7/1/3" and then fails on the
    // '/', leaving the triangle's other two indices -1 and unset: it cannot
    // load such files; this reader takes each token's vertex index.)
    int i(const std::string &t)
    {
        if (failed || t.empty())
            return failed = true, 0;
        char *end = nullptr;
        const long v = std::strtol(t.c_str(), &end, 10);
        if (end == t.c_str())
            return failed = true, 0;
        if (*end != '\0' && *end != '/')
            failed = true;
        return (int)v;
    }
};

}  // namespace

extern "C" int snch_obj_read(const char *path, float *verts, int64_t vert_capacity, int32_t *tris,
                             int64_t tri_capacity, int64_t *num_verts, int64_t *num_tris)
{
    if (!path || !num_verts || !num_tris)
        return snch::report_error(SNCH_ERR_INVALID_ARGUMENT, "path, num_verts and num_tris are required");
    if ((vert_capacity > 0 && !verts) || (tri_capacity > 0 && !tris))
        return snch::report_error(SNCH_ERR_INVALID_ARGUMENT, "a buffer with a capacity is NULL");
    FILE *fp = std::fopen(path, "rb");
    if (!fp)
        return snch::report_error(SNCH_ERR_INVALID_ARGUMENT, "Could not open .obj file.");
    int64_t nv = 0, nt = 0;
    std::string line;
    char buf[4096];
    bool more = true;
    while (more)
    {
        // one line (any length) without its '\n'
        line.clear();
        more = false;
        while (std::fgets(buf, sizeof buf, fp))
        {
            const size_t len = std::strlen(buf);
            if (len && buf[len - 1] == '\n')
            {
                line.append(buf, len - 1);
                more = true;
                break;
            }
            line.append(buf, len);
        }
        if (!more && line.empty())
            break;
        more = true;
        size_t pos = 0;
        const std::string prefix = token(line, &pos);
        Fields fl;
        if (prefix == "v")
        {
            const float x = fl.f(token(line, &pos));
            const float y = fl.f(token(line, &pos));
            const float z = fl.f(token(line, &pos));
            if (nv < vert_capacity)
            {
                verts[3 * nv] = x;
                verts[3 * nv + 1] = y;
                verts[3 * nv + 2] = z;
            }
            ++nv;
        }
        else if (prefix == "f")
        {
            const int a = fl.i(token(line, &pos));
            const int b = fl.i(token(line, &pos));
            const int c = fl.i(token(line, &pos));
            if (nt < tri_capacity)
            {
                tris[3 * nt] = a - 1;
                tris[3 * nt + 1] = b - 1;
                tris[3 * nt + 2] = c - 1;
            }
            ++nt;
        }
    }
    const bool err = std::ferror(fp) != 0;
    std::fclose(fp);
    if (err)
        return snch::report_error(SNCH_ERR_INVALID_ARGUMENT, std::string("read error on ") + path);
    *num_verts = nv;
    *num_tris = nt;
    return SNCH_OK;
}
