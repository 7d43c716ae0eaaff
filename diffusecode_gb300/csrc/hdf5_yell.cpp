// gen_hdf5_write (lib_f90/hdf_write.f90:12-326) as the output menu calls it
// for its 'hdf5' format (discus/prog/graphic.f90:604-635).  Datasets:
//   data            qval x out_scale over out_inc, H5T_NATIVE_DOUBLE, the
//                   dimensions (inc1, inc2, inc3) with the third index
//                   fastest; valmax > 0 scales the largest value to valmax
//   format          "Yell 1.0", a scalar variable-length string
//   is_direct       1 for the PDF values (qval 14 and 15), else 0; H5T_STD_I8BE
//   lower_limits    out_eck(:,1)                                H5T_IEEE_F64BE
//   step_sizes      out_vi(extr_abs,1), out_vi(extr_ord,2), out_vi(extr_top,3)
//   step_sizes_abs  out_vi(:,1); step_sizes_ord out_vi(:,2); _top out_vi(:,3)
//   unit_cell       cr_a0, cr_win
//   PROGRAM         "DISCUS60", one 9-byte null-terminated string
//
// The container is laid out from the HDF5 file format specification, with
// no HDF5 library: a version 0 superblock (8-byte offsets and lengths); the
// root group as a symbol table (a local heap of names, one version 1 B-tree
// node, one symbol table node with the names in byte order); per dataset a
// version 1 object header with dataspace (version 1; rank 0 is scalar),
// datatype (version 1), fill value (version 2) and contiguous layout
// (version 3) messages, its raw data in front of it; the string in a global
// heap collection.  These are the structures the library itself writes by
// default; its free-space and placement choices are not reproduced, so the
// bytes differ from the library's file while the objects and values agree.
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <map>
#include <string>
#include <vector>

#include "hdf5_yell.h"

namespace {

constexpr uint64_t UNDEF = ~0ull;       // the undefined address
constexpr int LEAF_K = 8;               // group leaf node K: 2K = 16 names per symbol table node
constexpr int NODE_K = 16;              // group internal node K: 2K children per B-tree node
constexpr uint64_t GCOL_SIZE = 4096;    // the smallest global heap collection
constexpr uint64_t HEAP_FREE_NULL = 1;  // "no next free block" in a local heap's free list

uint64_t pad8(uint64_t n) { return (n + 7) & ~7ull; }

uint64_t bits(double x)
{
    uint64_t u;
    memcpy(&u, &x, 8);
    return u;
}

// The file image; every structure starts on an 8-byte boundary.
struct Image {
    std::vector<uint8_t> b;
    uint64_t alloc(uint64_t n)
    {
        const uint64_t a = pad8(b.size());
        b.resize(a + n, 0);
        return a;
    }
    void le(uint64_t at, uint64_t v, int n)
    {
        for (int k = 0; k < n; k++) b[at + k] = (uint8_t)(v >> (8 * k));
    }
    void put(uint64_t at, const void *p, size_t n) { memcpy(&b[at], p, n); }
};

// Message data, little-endian fields
struct Enc {
    std::vector<uint8_t> d;
    Enc &u(uint64_t v, int n)
    {
        for (int k = 0; k < n; k++) d.push_back((uint8_t)(v >> (8 * k)));
        return *this;
    }
    Enc &cat(const Enc &e)
    {
        d.insert(d.end(), e.d.begin(), e.d.end());
        return *this;
    }
};

struct Msg {
    uint16_t type;
    uint8_t flags;   // bit 0: constant
    Enc e;
};

Msg dataspace(const std::vector<uint64_t> &dims)
{
    Enc e;
    e.u(1, 1).u(dims.size(), 1).u(0, 1).u(0, 1).u(0, 4);   // version 1, rank, no maximum dimensions
    for (uint64_t x : dims) e.u(x, 8);
    return {0x0001, 0, e};
}

// IEEE binary64: class 1; implied leading mantissa bit, sign at bit 63;
// offset 0, precision 64, exponent at 52 (11 bits), mantissa at 0 (52 bits), bias 1023
Enc f64_type(bool big_endian)
{
    Enc e;
    e.u(0x11, 1).u(0x20 | (big_endian ? 1 : 0), 1).u(63, 1).u(0, 1).u(8, 4);
    e.u(0, 2).u(64, 2).u(52, 1).u(11, 1).u(0, 1).u(52, 1).u(1023, 4);
    return e;
}

// One-byte integer: class 0; bit 0 byte order, bit 3 signed; offset 0, precision 8
Enc byte_type(bool big_endian, bool is_signed)
{
    Enc e;
    e.u(0x10, 1).u((big_endian ? 1 : 0) | (is_signed ? 8 : 0), 1).u(0, 1).u(0, 1).u(1, 4);
    e.u(0, 2).u(8, 2);
    return e;
}

// Fixed-length ASCII string, null terminated: class 3
Enc cstring_type(uint32_t size)
{
    Enc e;
    e.u(0x13, 1).u(0, 1).u(0, 1).u(0, 1).u(size, 4);
    return e;
}

// Variable-length ASCII string, null terminated: class 9 with type 1
// (string); 16 bytes per element (length, heap address, object index); the
// base type unsigned bytes
Enc vlstring_type()
{
    Enc e;
    e.u(0x19, 1).u(0x01, 1).u(0, 1).u(0, 1).u(16, 4);
    return e.cat(byte_type(false, false));
}

Msg datatype(const Enc &t) { return {0x0003, 1, t}; }

// Fill value, version 2: space allocated late, fill written if set, no fill value defined
Msg fill_value()
{
    Enc e;
    e.u(2, 1).u(2, 1).u(2, 1).u(0, 1);
    return {0x0005, 1, e};
}

// Data layout, version 3: contiguous at addr, size bytes
Msg layout(uint64_t addr, uint64_t size)
{
    Enc e;
    e.u(3, 1).u(1, 1).u(addr, 8).u(size, 8);
    return {0x0008, 0, e};
}

// A version 1 object header: version, reserved, message count, reference
// count, chunk size, 4 bytes to the 8-byte boundary, then per message type,
// size, flags, 3 reserved bytes and the data padded to 8 bytes.
uint64_t object_header(Image &f, const std::vector<Msg> &msgs)
{
    uint64_t chunk = 0;
    for (const Msg &m : msgs) chunk += 8 + pad8(m.e.d.size());
    const uint64_t at = f.alloc(16 + chunk);
    f.le(at, 1, 1);
    f.le(at + 2, msgs.size(), 2);
    f.le(at + 4, 1, 4);
    f.le(at + 8, chunk, 4);
    uint64_t p = at + 16;
    for (const Msg &m : msgs) {
        f.le(p, m.type, 2);
        f.le(p + 2, pad8(m.e.d.size()), 2);
        f.le(p + 4, m.flags, 1);
        if (!m.e.d.empty()) f.put(p + 8, m.e.d.data(), m.e.d.size());
        p += 8 + pad8(m.e.d.size());
    }
    return at;
}

// A dataset: its raw data, then its object header (returned)
uint64_t dataset(Image &f, const std::vector<uint64_t> &dims, const Enc &type, const std::vector<uint8_t> &raw)
{
    const uint64_t data = f.alloc(raw.size());
    if (!raw.empty()) f.put(data, raw.data(), raw.size());
    return object_header(f, {dataspace(dims), datatype(type), fill_value(), layout(data, raw.size())});
}

std::vector<uint8_t> f64_raw(const std::vector<double> &x, bool big_endian)
{
    std::vector<uint8_t> r(8 * x.size());
    for (size_t k = 0; k < x.size(); k++)
        for (int j = 0; j < 8; j++) r[8 * k + j] = (uint8_t)(bits(x[k]) >> (8 * (big_endian ? 7 - j : j)));
    return r;
}

}  // namespace

namespace dgpu_hdf5 {

int write_yell(const char *path, const dgpu_output *o, const double *v)
{
    const int64_t n1 = o->inc[0], n2 = o->inc[1], n3 = o->inc[2];
    const double scale = o->scale != 0.0 ? o->scale : 1.0;
    // values(k,j,i) = qvalues(i,j,k) (hdf_write.f90:117-133), times out_scale (graphic.f90:618)
    std::vector<double> vals((size_t)(n1 * n2 * n3));
    size_t l = 0;
    for (int64_t i = 0; i < n1; i++)
        for (int64_t j = 0; j < n2; j++)
            for (int64_t k = 0; k < n3; k++) vals[l++] = v[i + n1 * (j + n2 * k)] * scale;
    if (o->valmax > 0.0) {                     // hdf_write.f90:135-140, MAXVAL skipping NaN
        double mx = -HUGE_VAL;
        bool any = false;
        for (double x : vals)
            if (x == x) {
                mx = any ? fmax(mx, x) : x;
                any = true;
            }
        if (!any) mx = NAN;
        if (mx >= 0.0)
            for (double &x : vals) x = o->valmax * x / mx;
    }
    auto vi = [&](int r, int c) { return o->vi[(r - 1) + 3 * (c - 1)]; };

    std::vector<std::string> names = {"data",           "format",         "is_direct",      "lower_limits",
                                      "step_sizes",     "step_sizes_abs", "step_sizes_ord", "step_sizes_top",
                                      "unit_cell",      "PROGRAM"};
    std::sort(names.begin(), names.end());     // byte order, as the symbol table node is searched

    Image f;
    const uint64_t sb = f.alloc(96);
    const uint64_t root = object_header(f, {Msg{0x0011, 0, Enc().u(0, 8).u(0, 8)}});
    // the local heap: "" at 0, the names, then one 16-byte free block
    std::map<std::string, uint64_t> off;
    uint64_t seg = 8;
    for (const std::string &s : names) {
        off[s] = seg;
        seg += pad8(s.size() + 1);
    }
    const uint64_t free_at = seg;
    seg += 16;
    const uint64_t heap = f.alloc(32);
    const uint64_t heap_data = f.alloc(seg);
    f.put(heap, "HEAP", 4);
    f.le(heap + 8, seg, 8);
    f.le(heap + 16, free_at, 8);
    f.le(heap + 24, heap_data, 8);
    for (const std::string &s : names) f.put(heap_data + off[s], s.c_str(), s.size());
    f.le(heap_data + free_at, HEAP_FREE_NULL, 8);
    f.le(heap_data + free_at + 8, 16, 8);
    // the B-tree node: one symbol table node between "" and the last name
    const uint64_t tree = f.alloc(24 + 2 * NODE_K * 8 + (2 * NODE_K + 1) * 8);
    const uint64_t snod = f.alloc(8 + 2 * LEAF_K * 40);
    f.put(tree, "TREE", 4);
    f.le(tree + 6, 1, 2);
    f.le(tree + 8, UNDEF, 8);
    f.le(tree + 16, UNDEF, 8);
    f.le(tree + 24, 0, 8);
    f.le(tree + 32, snod, 8);
    f.le(tree + 40, off[names.back()], 8);
    // the root group's symbol table message
    f.le(root + 16 + 8, tree, 8);
    f.le(root + 16 + 16, heap, 8);

    // the global heap collection holding "Yell 1.0" as object 1
    const char *yell = "Yell 1.0";
    const uint64_t gcol = f.alloc(GCOL_SIZE);
    f.put(gcol, "GCOL", 4);
    f.le(gcol + 4, 1, 1);
    f.le(gcol + 8, GCOL_SIZE, 8);
    f.le(gcol + 16, 1, 2);
    f.le(gcol + 24, 8, 8);
    f.put(gcol + 32, yell, 8);
    f.le(gcol + 40, 0, 2);
    f.le(gcol + 48, GCOL_SIZE - 40, 8);

    std::map<std::string, uint64_t> hdr;
    hdr["data"] = dataset(f, {(uint64_t)n1, (uint64_t)n2, (uint64_t)n3}, f64_type(false), f64_raw(vals, false));
    {
        Enc r;
        r.u(8, 4).u(gcol, 8).u(1, 4);
        hdr["format"] = dataset(f, {}, vlstring_type(), r.d);
    }
    hdr["is_direct"] = dataset(f, {}, byte_type(true, true), {(uint8_t)(o->value == 14 || o->value == 15)});
    auto f64be = [&](const std::vector<double> &x) {
        return dataset(f, {(uint64_t)x.size()}, f64_type(true), f64_raw(x, true));
    };
    hdr["lower_limits"] = f64be({o->eck[0], o->eck[1], o->eck[2]});
    hdr["step_sizes"] = f64be({vi(o->extr_abs, 1), vi(o->extr_ord, 2), vi(o->extr_top, 3)});
    hdr["step_sizes_abs"] = f64be({vi(1, 1), vi(2, 1), vi(3, 1)});
    hdr["step_sizes_ord"] = f64be({vi(1, 2), vi(2, 2), vi(3, 2)});
    hdr["step_sizes_top"] = f64be({vi(1, 3), vi(2, 3), vi(3, 3)});
    hdr["unit_cell"] = f64be({o->a0[0], o->a0[1], o->a0[2], o->win[0], o->win[1], o->win[2]});
    {
        const char prog[9] = {'D', 'I', 'S', 'C', 'U', 'S', '6', '0', 0};
        hdr["PROGRAM"] = dataset(f, {1}, cstring_type(9), std::vector<uint8_t>(prog, prog + 9));
    }

    // the symbol table node: link name offset, object header address, no cache
    f.put(snod, "SNOD", 4);
    f.le(snod + 4, 1, 1);
    f.le(snod + 6, names.size(), 2);
    for (size_t k = 0; k < names.size(); k++) {
        f.le(snod + 8 + 40 * k, off[names[k]], 8);
        f.le(snod + 16 + 40 * k, hdr[names[k]], 8);
    }

    // the superblock, with the end-of-file address last
    const uint8_t sig[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
    f.put(sb, sig, 8);
    f.le(sb + 13, 8, 1);                        // size of offsets
    f.le(sb + 14, 8, 1);                        // size of lengths
    f.le(sb + 16, LEAF_K, 2);
    f.le(sb + 18, NODE_K, 2);
    f.le(sb + 24, 0, 8);                        // base address
    f.le(sb + 32, UNDEF, 8);                    // free-space info
    f.le(sb + 40, f.b.size(), 8);               // end of file
    f.le(sb + 48, UNDEF, 8);                    // driver information
    f.le(sb + 56, 0, 8);                        // root entry: name offset,
    f.le(sb + 64, root, 8);                     // object header,
    f.le(sb + 72, 1, 4);                        // cache type 1: B-tree and heap addresses
    f.le(sb + 80, tree, 8);
    f.le(sb + 88, heap, 8);

    FILE *fp = fopen(path, "wb");
    if (!fp) return DGPU_ERR_IO;
    const bool ok = fwrite(f.b.data(), 1, f.b.size(), fp) == f.b.size();
    return (fclose(fp) == 0 && ok) ? DGPU_OK : DGPU_ERR_IO;
}

}  // namespace dgpu_hdf5
