// gadget2.cpp -- format-II snapshot reader (see gadget2.h).
#include "gadget2.h"

#include <cstdio>
#include <cstring>
#include <memory>
#include <stdexcept>

namespace g2 {
namespace {

struct FileCloser {
    void operator()(FILE *f) const
    {
        if (f)
            fclose(f);
    }
};
using FilePtr = std::unique_ptr<FILE, FileCloser>;

[[noreturn]] void bad(const std::string &path, const std::string &what)
{
    throw std::runtime_error(path + ": " + what);
}

uint32_t bswap32(uint32_t v)
{
    return (v >> 24) | ((v >> 8) & 0xff00u) | ((v << 8) & 0xff0000u) | (v << 24);
}

// A 4-byte record marker, byte-swapped when the file's byte order differs.
bool read_marker(FILE *f, bool swap, uint32_t *out)
{
    uint32_t v;
    if (fread(&v, 4, 1, f) != 1)
        return false;
    *out = swap ? bswap32(v) : v;
    return true;
}

template <typename T>
T field(const unsigned char *b, size_t off, bool swap)
{
    unsigned char tmp[sizeof(T)];
    memcpy(tmp, b + off, sizeof(T));
    if (swap)
        for (size_t i = 0; i < sizeof(T) / 2; i++)
            std::swap(tmp[i], tmp[sizeof(T) - 1 - i]);
    T v;
    memcpy(&v, tmp, sizeof(T));
    return v;
}

// The 256-byte HEAD block, field offsets of the Gadget-2 io_header.
Header parse_header(const unsigned char *b, bool swap)
{
    Header h;
    for (int t = 0; t < kTypes; t++) {
        h.npart[t] = field<uint32_t>(b, 4 * t, swap);
        h.mass[t] = field<double>(b, 24 + 8 * t, swap);
        h.npart_total[t] = field<uint32_t>(b, 96 + 4 * t, swap);
        h.npart_total_hw[t] = field<uint32_t>(b, 168 + 4 * t, swap);
    }
    h.time = field<double>(b, 72, swap);
    h.redshift = field<double>(b, 80, swap);
    h.num_files = field<int32_t>(b, 124, swap);
    h.box = field<double>(b, 128, swap);
    h.omega0 = field<double>(b, 136, swap);
    h.omega_lambda = field<double>(b, 144, swap);
    h.hubble = field<double>(b, 152, swap);
    return h;
}

struct Indexed {
    File file;
    bool swap = false;
};

// Walk the label and data records of one file.
Indexed index_file(const std::string &path)
{
    FilePtr f(fopen(path.c_str(), "rb"));
    if (!f)
        bad(path, "cannot open");
    Indexed out;
    out.file.path = path;
    uint32_t first;
    if (!read_marker(f.get(), false, &first))
        bad(path, "empty file");
    if (first == 8u) {
        out.swap = false;
    } else if (bswap32(first) == 8u) {
        out.swap = true;
    } else {
        bad(path, "not a format-II snapshot (first record is " + std::to_string(first) +
                      " bytes, a block label has 8)");
    }
    fseek(f.get(), 0, SEEK_SET);
    std::vector<unsigned char> head;
    for (;;) {
        uint32_t m1;
        if (!read_marker(f.get(), out.swap, &m1))
            break;  // end of file
        char name[5] = {0};
        uint32_t skip, m2;
        if (m1 != 8u || fread(name, 1, 4, f.get()) != 4 || !read_marker(f.get(), out.swap, &skip) ||
            !read_marker(f.get(), out.swap, &m2) || m2 != 8u)
            bad(path, "corrupt block label");
        uint32_t s1, s2;
        if (!read_marker(f.get(), out.swap, &s1))
            bad(path, std::string("block ") + name + " has no data record");
        const int64_t off = ftell(f.get());
        if (std::string(name) == "HEAD") {
            head.resize(s1);
            if (fread(head.data(), 1, s1, f.get()) != s1)
                bad(path, "short HEAD block");
        } else if (fseek(f.get(), (long)s1, SEEK_CUR) != 0) {
            bad(path, std::string("short block ") + name);
        }
        if (!read_marker(f.get(), out.swap, &s2) || s1 != s2)
            bad(path, std::string("record markers of block ") + name + " disagree");
        Block b;
        b.offset = off;
        b.size = s1;
        out.file.blocks.emplace_back(std::string(name), b);
    }
    if (head.size() < 256)
        bad(path, "no 256-byte HEAD block");
    out.file.head = parse_header(head.data(), out.swap);
    return out;
}

bool exists(const std::string &p)
{
    FilePtr f(fopen(p.c_str(), "rb"));
    return (bool)f;
}

int64_t before(const Header &h, int type, bool masses_only)
{
    int64_t n = 0;
    for (int t = 0; t < type; t++)
        if (!masses_only || h.mass[t] == 0.0)
            n += h.npart[t];
    return n;
}

}  // namespace

const Block *File::find(const std::string &name) const
{
    for (const auto &kv : blocks)
        if (kv.first == name)
            return &kv.second;
    return nullptr;
}

Snapshot::Snapshot(const std::string &base)
{
    std::vector<Indexed> idx;
    if (exists(base)) {
        idx.push_back(index_file(base));
    } else if (exists(base + ".0")) {
        idx.push_back(index_file(base + ".0"));
        const int nf = idx[0].file.head.num_files;
        for (int i = 1; i < nf; i++)
            idx.push_back(index_file(base + "." + std::to_string(i)));
    } else {
        bad(base, "no such snapshot (neither the file nor " + base + ".0 exists)");
    }
    for (auto &x : idx) {
        if (x.swap)
            bad(x.file.path, "opposite byte order: not supported");
        const Header &h = x.file.head;
        int64_t all = 0, with_mass = 0;
        for (int t = 0; t < kTypes; t++) {
            all += h.npart[t];
            with_mass += h.mass[t] == 0.0 ? h.npart[t] : 0;
        }
        const Block *pos = x.file.find("POS ");
        if (all > 0) {
            if (!pos)
                bad(x.file.path, "no POS block");
            if (pos->size == 24 * all)
                bad(x.file.path, "positions are stored as double: 24 bytes per particle, "
                                 "this reader takes 12 (float)");
            if (pos->size != 12 * all)
                bad(x.file.path, "POS block of " + std::to_string(pos->size) + " bytes for " +
                                     std::to_string(all) + " particles");
        }
        const Block *mb = x.file.find("MASS");
        if (with_mass > 0 && (!mb || mb->size != 4 * with_mass))
            bad(x.file.path, "MASS block missing or not 4 bytes per particle of the types "
                             "without a header mass");
        files_.push_back(x.file);
    }
}

int64_t Snapshot::npart(int type) const
{
    int64_t n = 0;
    for (const auto &f : files_)
        n += f.head.npart[type];
    return n;
}

void Snapshot::read(int type, int64_t start, int64_t n, float *pos, float *m) const
{
    int64_t first = 0;  // index of this file's first particle of `type`
    int64_t done = 0;
    for (const auto &f : files_) {
        const int64_t here = f.head.npart[type];
        const int64_t lo = std::max<int64_t>(start + done, first);
        const int64_t hi = std::min<int64_t>(start + n, first + here);
        if (lo < hi) {
            FilePtr fp(fopen(f.path.c_str(), "rb"));
            if (!fp)
                bad(f.path, "cannot reopen");
            const int64_t k = hi - lo, i0 = lo - first;
            const Block *pb = f.find("POS ");
            const int64_t po = pb->offset + 12 * (before(f.head, type, false) + i0);
            if (fseek(fp.get(), (long)po, SEEK_SET) != 0 ||
                fread(pos + 3 * done, 12, (size_t)k, fp.get()) != (size_t)k)
                bad(f.path, "short read of POS");
            if (f.head.mass[type] == 0.0 && m) {
                const Block *mb = f.find("MASS");
                const int64_t mo = mb->offset + 4 * (before(f.head, type, true) + i0);
                if (fseek(fp.get(), (long)mo, SEEK_SET) != 0 ||
                    fread(m + done, 4, (size_t)k, fp.get()) != (size_t)k)
                    bad(f.path, "short read of MASS");
            }
            done += k;
        }
        first += here;
        if (done == n)
            break;
    }
    if (done != n)
        throw std::runtime_error("read past the last particle of type " + std::to_string(type));
}

}  // namespace g2
