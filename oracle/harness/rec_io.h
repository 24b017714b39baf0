// Tiny named-array record format shared by the oracle harness and the fixture
// scripts (test infrastructure only).
//
// A file is a sequence of records:
//   char name[32] (NUL padded) | char dtype ('d' = f64, 'i' = i64) | int32 ndim |
//   int64 shape[ndim] | payload (row-major, little endian)
#ifndef BIB_ORACLE_REC_IO_H
#define BIB_ORACLE_REC_IO_H
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <vector>

namespace recio {

struct Array {
    char dtype;
    std::vector<long long> shape;
    std::vector<double> d;
    std::vector<long long> i;
    size_t size() const {
        size_t n = 1;
        for (size_t k = 0; k < shape.size(); ++k) n *= (size_t)shape[k];
        return n;
    }
};

typedef std::map<std::string, Array> Bundle;

inline Bundle read_file(const char* path) {
    Bundle b;
    FILE* f = std::fopen(path, "rb");
    if (!f) { std::fprintf(stderr, "cannot open %s\n", path); std::exit(2); }
    for (;;) {
        char name[33];
        std::memset(name, 0, sizeof(name));
        if (std::fread(name, 1, 32, f) != 32) break;
        Array a;
        int nd = 0;
        if (std::fread(&a.dtype, 1, 1, f) != 1 || std::fread(&nd, 4, 1, f) != 1) break;
        a.shape.resize(nd);
        if (nd && std::fread(&a.shape[0], 8, nd, f) != (size_t)nd) break;
        size_t n = a.size();
        if (a.dtype == 'd') {
            a.d.resize(n);
            if (n && std::fread(&a.d[0], 8, n, f) != n) break;
        } else {
            a.i.resize(n);
            if (n && std::fread(&a.i[0], 8, n, f) != n) break;
        }
        b[std::string(name)] = a;
    }
    std::fclose(f);
    return b;
}

inline void write_record(FILE* f, const std::string& name, char dtype, const std::vector<long long>& shape,
                         const void* data) {
    char nm[32];
    std::memset(nm, 0, 32);
    std::strncpy(nm, name.c_str(), 31);
    std::fwrite(nm, 1, 32, f);
    std::fwrite(&dtype, 1, 1, f);
    int nd = (int)shape.size();
    std::fwrite(&nd, 4, 1, f);
    size_t n = 1;
    for (int k = 0; k < nd; ++k) n *= (size_t)shape[k];
    if (nd) std::fwrite(&shape[0], 8, nd, f);
    if (n) std::fwrite(data, 8, n, f);
}

inline const Array& need(const Bundle& b, const char* name) {
    Bundle::const_iterator it = b.find(name);
    if (it == b.end()) { std::fprintf(stderr, "missing input %s\n", name); std::exit(2); }
    return it->second;
}
inline double num(const Bundle& b, const char* name) {
    const Array& a = need(b, name);
    return a.dtype == 'd' ? a.d[0] : (double)a.i[0];
}
inline long long inum(const Bundle& b, const char* name) {
    const Array& a = need(b, name);
    return a.dtype == 'i' ? a.i[0] : (long long)a.d[0];
}
inline bool has(const Bundle& b, const char* name) { return b.find(name) != b.end(); }

struct Writer {
    FILE* f;
    explicit Writer(const char* path) : f(std::fopen(path, "wb")) {
        if (!f) { std::fprintf(stderr, "cannot write %s\n", path); std::exit(2); }
    }
    ~Writer() { std::fclose(f); }
    void d(const std::string& name, const std::vector<long long>& shape, const std::vector<double>& v) {
        write_record(f, name, 'd', shape, v.empty() ? 0 : &v[0]);
    }
    void i(const std::string& name, const std::vector<long long>& shape, const std::vector<long long>& v) {
        write_record(f, name, 'i', shape, v.empty() ? 0 : &v[0]);
    }
};

inline std::vector<long long> shp(long long a) { std::vector<long long> s(1, a); return s; }
inline std::vector<long long> shp(long long a, long long b) { std::vector<long long> s; s.push_back(a); s.push_back(b); return s; }
inline std::vector<long long> shp(long long a, long long b, long long c) { std::vector<long long> s = shp(a, b); s.push_back(c); return s; }
inline std::vector<long long> shp(long long a, long long b, long long c, long long d) { std::vector<long long> s = shp(a, b, c); s.push_back(d); return s; }

}  // namespace recio
#endif
