// bigfile.cpp -- BigFile snapshot reader (layout in bigfile.h).
#include "bigfile.h"

#include <sys/stat.h>

#include <cstdio>
#include <cstring>
#include <fstream>
#include <sstream>
#include <stdexcept>

namespace bigfile {
namespace {

[[noreturn]] void fail(const std::string &msg)
{
    throw std::runtime_error("BigFile: " + msg);
}

bool is_dir(const std::string &p)
{
    struct stat st;
    return stat(p.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

bool host_little_endian()
{
    const uint16_t one = 1;
    unsigned char b;
    std::memcpy(&b, &one, 1);
    return b == 1;
}

// Parse a dtype string such as "<f8", "=i4" or "|u1".
void parse_dtype(const std::string &d, char *order, char *kind, int *size)
{
    if (d.size() < 3 || std::strchr("<>=|", d[0]) == nullptr || std::strchr("fiu", d[1]) == nullptr)
        fail("unsupported dtype '" + d + "'");
    *order = d[0];
    *kind = d[1];
    *size = std::atoi(d.c_str() + 2);
    const bool ok = (*kind == 'f') ? (*size == 4 || *size == 8)
                                   : (*size == 1 || *size == 2 || *size == 4 || *size == 8);
    if (!ok)
        fail("unsupported dtype '" + d + "'");
}

// One item at `p` (in `order`) as double.
double item(const unsigned char *p, char order, char kind, int size)
{
    unsigned char b[8];
    const bool swap = (order == '>' && host_little_endian()) || (order == '<' && !host_little_endian());
    for (int k = 0; k < size; k++)
        b[k] = swap ? p[size - 1 - k] : p[k];
    if (kind == 'f') {
        if (size == 4) {
            float v;
            std::memcpy(&v, b, 4);
            return (double)v;
        }
        double v;
        std::memcpy(&v, b, 8);
        return v;
    }
    uint64_t u = 0;
    for (int k = 0; k < size; k++)  // assembled little-endian after the swap
        u |= (uint64_t)b[host_little_endian() ? k : size - 1 - k] << (8 * k);
    if (kind == 'u')
        return (double)u;
    const int bits = 8 * size;
    const int64_t s = bits == 64 ? (int64_t)u : (int64_t)(u << (64 - bits)) >> (64 - bits);
    return (double)s;
}

int hexval(char c)
{
    if (c >= '0' && c <= '9')
        return c - '0';
    if (c >= 'a' && c <= 'f')
        return c - 'a' + 10;
    if (c >= 'A' && c <= 'F')
        return c - 'A' + 10;
    return -1;
}

}  // namespace

Column open_column(const std::string &snapshot, const std::string &name)
{
    Column c;
    c.dir = snapshot + "/" + name;
    std::ifstream h(c.dir + "/header");
    if (!h)
        fail("no block '" + name + "' in " + snapshot);
    std::string key, dtype;
    int64_t nfile = -1;
    while (h >> key) {
        if (key == "DTYPE:") {
            h >> dtype;
        } else if (key == "NMEMB:") {
            h >> c.nmemb;
        } else if (key == "NFILE:") {
            h >> nfile;
            break;
        } else {
            fail("unexpected '" + key + "' in " + c.dir + "/header");
        }
    }
    if (dtype.empty() || nfile < 0 || c.nmemb < 1)
        fail("incomplete header of block '" + name + "'");
    parse_dtype(dtype, &c.order, &c.kind, &c.size);
    std::string line;
    std::getline(h, line);  // rest of the NFILE line
    for (int64_t f = 0; f < nfile; f++) {
        if (!std::getline(h, line))
            fail("block '" + name + "' lists fewer data files than NFILE");
        unsigned fid = 0;
        long long rows = -1;
        unsigned ck = 0, sv = 0;
        if (std::sscanf(line.c_str(), " %X: %lld : %u : %u", &fid, &rows, &ck, &sv) < 2 ||
            fid != (unsigned)f || rows < 0)
            fail("bad data-file line '" + line + "' in block '" + name + "'");
        c.file_rows.push_back(rows);
        c.rows += rows;
    }
    return c;
}

std::map<std::string, Attr> read_attrs(const std::string &block_dir)
{
    std::map<std::string, Attr> out;
    std::ifstream f(block_dir + "/attr-v2");
    if (!f)
        fail("no attr-v2 file in " + block_dir);
    std::string line;
    while (std::getline(f, line)) {
        std::istringstream ss(line);
        std::string name, dtype, hex;
        int64_t nmemb = 0;
        if (!(ss >> name >> dtype >> nmemb >> hex))
            continue;
        char order, kind;
        int size;
        parse_dtype(dtype, &order, &kind, &size);
        if ((int64_t)hex.size() != 2 * nmemb * size)
            fail("attribute '" + name + "' has " + std::to_string(hex.size() / 2) +
                 " bytes for " + std::to_string(nmemb) + " x " + dtype);
        std::vector<unsigned char> bytes(hex.size() / 2);
        for (size_t k = 0; k < bytes.size(); k++) {
            const int hi = hexval(hex[2 * k]), lo = hexval(hex[2 * k + 1]);
            if (hi < 0 || lo < 0)
                fail("attribute '" + name + "' is not hexadecimal");
            bytes[k] = (unsigned char)(16 * hi + lo);
        }
        Attr a;
        a.dtype = dtype;
        for (int64_t k = 0; k < nmemb; k++) {
            const double v = item(bytes.data() + k * size, order, kind, size);
            a.f.push_back(v);
            a.i.push_back((int64_t)v);
        }
        if (kind != 'f' && size == 8) {  // keep 64-bit integers exact
            for (int64_t k = 0; k < nmemb; k++) {
                uint64_t u = 0;
                for (int b = 0; b < 8; b++) {
                    const int src = (order == '>') ? 7 - b : b;
                    u |= (uint64_t)bytes[(size_t)(k * 8 + src)] << (8 * b);
                }
                a.i[(size_t)k] = (int64_t)u;
            }
        }
        out[name] = a;
    }
    return out;
}

void read_rows(const Column &c, int64_t start, int64_t n, double *out)
{
    if (start < 0 || n < 0 || start + n > c.rows)
        fail("rows [" + std::to_string(start) + ", " + std::to_string(start + n) +
             ") outside block " + c.dir);
    const int64_t row_bytes = (int64_t)c.size * c.nmemb;
    std::vector<unsigned char> buf;
    int64_t first = 0;  // first row of file f
    for (size_t f = 0; f < c.file_rows.size() && n > 0; f++) {
        const int64_t rows = c.file_rows[f];
        if (start >= first + rows) {
            first += rows;
            continue;
        }
        const int64_t off = start - first;
        const int64_t take = std::min(n, rows - off);
        char name[16];
        std::snprintf(name, sizeof name, "%06X", (unsigned)f);
        const std::string path = c.dir + "/" + name;
        FILE *fp = std::fopen(path.c_str(), "rb");
        if (!fp)
            fail("cannot open " + path);
        buf.resize((size_t)(take * row_bytes));
        const bool ok = fseeko(fp, (off_t)(off * row_bytes), SEEK_SET) == 0 &&
                        std::fread(buf.data(), 1, buf.size(), fp) == buf.size();
        std::fclose(fp);
        if (!ok)
            fail("short read from " + path);
        const int64_t items = take * c.nmemb;
        for (int64_t k = 0; k < items; k++)
            out[k] = item(buf.data() + k * c.size, c.order, c.kind, c.size);
        out += items;
        start += take;
        n -= take;
        first += rows;
    }
    if (n > 0)
        fail("block " + c.dir + " holds fewer rows than its header lists");
}

bool Snapshot::is_bigfile(const std::string &dir)
{
    if (!is_dir(dir))
        return false;
    try {
        open_column(dir, "Header");
        return true;
    } catch (const std::exception &) {
        return false;
    }
}

Snapshot::Snapshot(const std::string &dir) : dir_(dir)
{
    if (!is_dir(dir))
        fail("no such snapshot directory: " + dir);
    open_column(dir, "Header");
    const auto attrs = read_attrs(dir + "/Header");
    auto get = [&](const char *name, size_t count) -> const Attr & {
        auto it = attrs.find(name);
        if (it == attrs.end() || it->second.f.size() != count)
            fail(std::string("Header attribute ") + name + " missing or of the wrong length");
        return it->second;
    };
    const Attr &np = get("TotNumPart", 6), &mt = get("MassTable", 6);
    for (int t = 0; t < 6; t++) {
        npart_[t] = np.i[(size_t)t];
        mass_[t] = mt.f[(size_t)t];
    }
    time_ = get("Time", 1).f[0];
    hubble_ = get("HubbleParam", 1).f[0];
    omega0_ = get("Omega0", 1).f[0];
    box_ = get("BoxSize", 1).f[0];
}

void Snapshot::read(int type, int64_t start, int64_t n, float *pos, float *m) const
{
    const Column p = open_column(dir_, std::to_string(type) + "/Position");
    if (p.nmemb != 3)
        fail("Position of type " + std::to_string(type) + " does not have 3 members");
    std::vector<double> tmp((size_t)(3 * n));
    read_rows(p, start, n, tmp.data());
    for (int64_t k = 0; k < 3 * n; k++)
        pos[k] = (float)tmp[(size_t)k];
    if (mass_[type] == 0.0 && m) {
        const Column mc = open_column(dir_, std::to_string(type) + "/Mass");
        tmp.resize((size_t)n);
        read_rows(mc, start, n, tmp.data());
        for (int64_t k = 0; k < n; k++)
            m[k] = (float)tmp[(size_t)k];
    }
}

}  // namespace bigfile
