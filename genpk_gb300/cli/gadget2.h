// gadget2.h -- minimal reader for Gadget-2 format-II snapshots (single file or
// a set base.0, base.1, ...), enough for the power-spectrum driver: the header,
// and the POS and MASS blocks of one particle type in chunks.
//
// The reference reads snapshots through GadgetReader (GSnap), a git submodule
// that is not part of its tree; its read_fieldize (read_fieldize.cpp:17-97)
// uses GetNpart, GetHeader().mass/BoxSize, GetBlock("POS ") and
// GetBlock("MASS") with a skip-type mask.  This reader provides those
// operations for the format-II layout:
//   every block is a label record {int32 8, char name[4], int32 size + 8,
//   int32 8} followed by a data record {int32 size, data, int32 size};
//   HEAD is 256 bytes (npart[6], mass[6], time, redshift, ..., npartTotal[6],
//   ..., num_files, BoxSize, Omega0, OmegaLambda, HubbleParam, ...,
//   npartTotalHighWord[6]); POS holds float[3] per particle, types in order;
//   MASS holds one float per particle of the types whose header mass is 0.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace g2 {

constexpr int kTypes = 6;

struct Header {
    uint32_t npart[kTypes] = {};        // in this file
    double mass[kTypes] = {};           // 0: per-particle masses in the MASS block
    double time = 0.0;                  // scale factor
    double redshift = 0.0;
    uint32_t npart_total[kTypes] = {};  // low words of the whole snapshot's counts
    int32_t num_files = 1;
    double box = 0.0;
    double omega0 = 0.0, omega_lambda = 0.0, hubble = 0.0;
    uint32_t npart_total_hw[kTypes] = {};
};

struct Block {
    int64_t offset = -1;  // file offset of the data
    int64_t size = 0;     // bytes
};

struct File {
    std::string path;
    Header head;
    std::vector<std::pair<std::string, Block>> blocks;
    const Block *find(const std::string &name) const;
};

class Snapshot {
public:
    // `base`: a file name, or the base name of a set base.0 ... base.(n-1).
    // Throws std::runtime_error with a message on any format problem.
    explicit Snapshot(const std::string &base);

    const Header &header() const { return files_[0].head; }
    int num_files() const { return (int)files_.size(); }
    int64_t npart(int type) const;  // over all files
    double box() const { return files_[0].head.box; }
    double mass(int type) const { return files_[0].head.mass[type]; }

    // Particles [start, start + n) of `type` (counted over the files in
    // order): positions into pos[3n]; masses into m[n] when the type's header
    // mass is 0 (m may be null otherwise).
    void read(int type, int64_t start, int64_t n, float *pos, float *m) const;

private:
    std::vector<File> files_;
};

}  // namespace g2
