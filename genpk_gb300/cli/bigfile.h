// bigfile.h -- reader for BigFile snapshots (the format of MP-Gadget), enough
// for the power-spectrum driver: the Header block's attributes and the
// "<type>/Position" and "<type>/Mass" columns in chunks.
//
// The reference reads BigFile through the bigfile library, a git submodule
// that is not part of its tree; read_fieldize_bigfile.cpp:7-126 opens the
// "Header" block, reads its attributes TotNumPart (u8[6]), MassTable (f8[6]),
// Time, HubbleParam, Omega0 and BoxSize (f8), the column "<type>/Position" as
// f8[3] narrowed to float, and "<type>/Mass" as f4 where MassTable[type] is 0.
// This reader follows the library's published on-disk layout:
//   a snapshot is a directory, and every block (column) a directory below it;
//   a block directory holds a text file "header":
//       DTYPE: <dtype>      e.g. <f8: byte order (< little, > big, = native,
//                           | none) then kind (f, i, u) and item size
//       NMEMB: <members per row>
//       NFILE: <data files>
//   followed by one line per data file, "%06X: rows : checksum : sysv-sum";
//   the rows themselves are raw binary in data files named "%06X" (000000,
//   000001, ...), in order; and attributes in a text file "attr-v2", one per
//   line: "name dtype nmemb hex-bytes #HUMANE [ ... ]".
#pragma once

#include <cstdint>
#include <map>
#include <string>
#include <vector>

namespace bigfile {

struct Column {
    std::string dir;
    char order = '<';   // byte order of the data
    char kind = 'f';    // f, i or u
    int size = 8;       // bytes per item
    int nmemb = 1;      // items per row
    std::vector<int64_t> file_rows;
    int64_t rows = 0;
};

// A typed attribute: its values as double (floating point) and as int64 (integers).
struct Attr {
    std::string dtype;
    std::vector<double> f;
    std::vector<int64_t> i;
};

class Snapshot {
public:
    // Opens the snapshot directory and its Header block.  Throws
    // std::runtime_error with a message on any format problem.
    explicit Snapshot(const std::string &dir);

    // True when `dir` is a directory holding a readable Header block.
    static bool is_bigfile(const std::string &dir);

    int64_t npart(int type) const { return npart_[type]; }
    double mass(int type) const { return mass_[type]; }
    double box() const { return box_; }
    double time() const { return time_; }
    double hubble() const { return hubble_; }
    double omega0() const { return omega0_; }

    // Particles [start, start + n) of `type`: positions into pos[3n] (read as
    // double, narrowed to float, as the reference does), masses into m[n] as
    // float when the type's MassTable entry is 0 (m may be null otherwise).
    void read(int type, int64_t start, int64_t n, float *pos, float *m) const;

private:
    std::string dir_;
    int64_t npart_[6] = {};
    double mass_[6] = {};
    double box_ = 0.0, time_ = 0.0, hubble_ = 0.0, omega0_ = 0.0;
};

// Lower-level pieces, exposed for the reader's tests.
Column open_column(const std::string &snapshot, const std::string &name);
std::map<std::string, Attr> read_attrs(const std::string &block_dir);
// Rows [start, start + n) of a column, every item converted to double.
void read_rows(const Column &c, int64_t start, int64_t n, double *out);

}  // namespace bigfile
