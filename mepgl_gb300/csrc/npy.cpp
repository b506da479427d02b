// npy.cpp -- see npy.h.  Little-endian hosts only (x86-64, AArch64).
#include "npy.h"

#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace npy {

size_t Array::count() const
{
    size_t n = 1;
    for (size_t s : shape) n *= s;
    return n;
}

namespace {

std::string field(const std::string &h, const std::string &key)
{
    const size_t k = h.find("'" + key + "'");
    if (k == std::string::npos) return "";
    size_t c = h.find(':', k);
    if (c == std::string::npos) return "";
    ++c;
    while (c < h.size() && h[c] == ' ') ++c;
    if (h[c] == '\'') {
        const size_t e = h.find('\'', c + 1);
        return h.substr(c + 1, e - c - 1);
    }
    if (h[c] == '(') {
        const size_t e = h.find(')', c);
        return h.substr(c + 1, e - c - 1);
    }
    size_t e = c;
    while (e < h.size() && h[e] != ',' && h[e] != '}') ++e;
    return h.substr(c, e - c);
}

size_t itemsize(const std::string &d)
{
    if (d.size() < 3) return 0;
    return (size_t)std::stoul(d.substr(2));
}

template <class T>
void write_impl(const std::string &path, const T *data, const std::vector<size_t> &shape, const char *descr)
{
    std::ostringstream dict;
    dict << "{'descr': '" << descr << "', 'fortran_order': False, 'shape': (";
    for (size_t i = 0; i < shape.size(); ++i) dict << shape[i] << (shape.size() == 1 || i + 1 < shape.size() ? "," : "");
    dict << "), }";
    std::string h = dict.str();
    const size_t pre = 10;   // magic(6) + version(2) + len(2)
    size_t total = pre + h.size() + 1;
    const size_t pad = (64 - total % 64) % 64;
    h.append(pad, ' ');
    h.push_back('\n');
    std::ofstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot write " + path);
    const char magic[8] = {'\x93', 'N', 'U', 'M', 'P', 'Y', 1, 0};
    f.write(magic, 8);
    const uint16_t len = (uint16_t)h.size();
    f.write((const char *)&len, 2);
    f.write(h.data(), h.size());
    size_t n = 1;
    for (size_t s : shape) n *= s;
    f.write((const char *)data, n * sizeof(T));
    if (!f) throw std::runtime_error("short write " + path);
}

}  // namespace

Array read(const std::string &path)
{
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open " + path);
    char magic[8];
    f.read(magic, 8);
    if (!f || std::memcmp(magic, "\x93NUMPY", 6) != 0) throw std::runtime_error("not an .npy file: " + path);
    uint32_t hlen = 0;
    if (magic[6] == 1) {
        uint16_t l;
        f.read((char *)&l, 2);
        hlen = l;
    } else {
        f.read((char *)&hlen, 4);
    }
    std::string h(hlen, '\0');
    f.read(&h[0], hlen);
    if (!f) throw std::runtime_error("truncated header: " + path);
    Array a;
    a.descr = field(h, "descr");
    a.fortran = field(h, "fortran_order").find("True") != std::string::npos;
    std::string sh = field(h, "shape");
    std::stringstream ss(sh);
    std::string tok;
    while (std::getline(ss, tok, ',')) {
        size_t b = tok.find_first_not_of(' ');
        if (b == std::string::npos) continue;
        a.shape.push_back((size_t)std::stoull(tok.substr(b)));
    }
    if (a.descr.empty() || (a.descr[0] != '<' && a.descr[0] != '|'))
        throw std::runtime_error("unsupported byte order '" + a.descr + "' in " + path);
    const size_t nbytes = a.count() * itemsize(a.descr);
    a.bytes.resize(nbytes);
    f.read(a.bytes.data(), nbytes);
    if ((size_t)f.gcount() != nbytes) throw std::runtime_error("truncated data: " + path);
    return a;
}

std::vector<double> as_double(const Array &a)
{
    if (a.fortran) throw std::runtime_error("fortran-ordered arrays are not supported");
    const size_t n = a.count();
    std::vector<double> out(n);
    const std::string t = a.descr.substr(1);
    const char *p = a.bytes.data();
    for (size_t i = 0; i < n; ++i) {
        if (t == "f8") { double v; std::memcpy(&v, p + 8 * i, 8); out[i] = v; }
        else if (t == "f4") { float v; std::memcpy(&v, p + 4 * i, 4); out[i] = v; }
        else if (t == "i4") { int32_t v; std::memcpy(&v, p + 4 * i, 4); out[i] = v; }
        else if (t == "i8") { int64_t v; std::memcpy(&v, p + 8 * i, 8); out[i] = (double)v; }
        else if (t == "b1" || t == "u1") out[i] = (unsigned char)p[i];
        else throw std::runtime_error("unsupported dtype " + a.descr);
    }
    return out;
}

std::vector<int32_t> as_int32(const Array &a)
{
    const std::vector<double> d = as_double(a);
    std::vector<int32_t> out(d.size());
    for (size_t i = 0; i < d.size(); ++i) out[i] = (int32_t)d[i];
    return out;
}

void write(const std::string &path, const double *data, const std::vector<size_t> &shape)
{
    write_impl(path, data, shape, "<f8");
}
void write(const std::string &path, const float *data, const std::vector<size_t> &shape)
{
    write_impl(path, data, shape, "<f4");
}
void write(const std::string &path, const int32_t *data, const std::vector<size_t> &shape)
{
    write_impl(path, data, shape, "<i4");
}

}  // namespace npy
