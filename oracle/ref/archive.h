// Tensor archive of the fixture harnesses (test infrastructure only):
// "ASTG" u32 count, then per entry: u32 namelen, name, u8 dtype (0 f64, 1 i32, 2 i64, 3 u8),
// u32 ndim, u64 dims[ndim], raw little-endian data.  Read by tests/golden/astg_archive.py.
#pragma once
#include <cstdint>
#include <cstring>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace fixture {

struct Archive {
    struct Entry {
        std::string name;
        uint8_t dtype;
        std::vector<uint64_t> dims;
        std::vector<char> bytes;
    };
    std::vector<Entry> entries;

    template <class T>
    void add(const std::string& name, uint8_t dtype, const std::vector<T>& v, std::vector<uint64_t> dims = {}) {
        Entry e;
        e.name = name;
        e.dtype = dtype;
        e.dims = dims.empty() ? std::vector<uint64_t>{(uint64_t)v.size()} : dims;
        e.bytes.resize(v.size() * sizeof(T));
        if (!v.empty()) memcpy(e.bytes.data(), v.data(), e.bytes.size());
        entries.push_back(std::move(e));
    }
    void f64(const std::string& n, const std::vector<double>& v, std::vector<uint64_t> d = {}) { add(n, 0, v, d); }
    void i32(const std::string& n, const std::vector<int32_t>& v, std::vector<uint64_t> d = {}) { add(n, 1, v, d); }
    void i64(const std::string& n, const std::vector<int64_t>& v, std::vector<uint64_t> d = {}) { add(n, 2, v, d); }
    void u8(const std::string& n, const std::vector<uint8_t>& v, std::vector<uint64_t> d = {}) { add(n, 3, v, d); }

    void write(const std::string& path) const {
        std::ofstream out(path, std::ios::binary);
        if (!out) throw std::runtime_error("cannot open " + path);
        out.write("ASTG", 4);
        uint32_t n = entries.size();
        out.write((const char*)&n, 4);
        for (auto& e : entries) {
            uint32_t l = e.name.size();
            out.write((const char*)&l, 4);
            out.write(e.name.data(), l);
            out.write((const char*)&e.dtype, 1);
            uint32_t nd = e.dims.size();
            out.write((const char*)&nd, 4);
            out.write((const char*)e.dims.data(), 8 * nd);
            out.write(e.bytes.data(), e.bytes.size());
        }
    }
};

}  // namespace fixture
