// gen_pk_gb300.cpp -- the gen-pk command line on the GB300 library.
//
// Same flags, files and flow as the reference driver (gen-pk.cpp:72-367):
//   -i snapshot   a BigFile snapshot directory (bigfile.h), else a format-II
//                 file or the base name of a set base.0, base.1, ...
//                 (gen-pk.cpp:121-152 tries HDF5, then BigFile, then Gadget;
//                 HDF5 files are recognised and refused: libhdf5 is absent)
//   -o outdir     one file per particle type: outdir/PK-<type>-<input>
//   -j snapshot2  cross spectrum of each type between the two snapshots:
//                 outdir/PX-<type>-<input>   (gen-pk.cpp:240-303)
//   -c type       cross spectrum of DM (type 1) with `type` in the -i snapshot:
//                 outdir/PK-DMx<type>-<input>   (gen-pk.cpp:304-356)
//   -s 1          stars (type 4) are added to the baryon (type 0) field
//   -h            usage
// and three additions: -g N (grid), -b B (log-k bins) override the reference's
// rule N = max over types of min(2 nexttwo(cbrt(npart)), 3072), B = N
// (gen-pk.cpp:169-173); -d prints the snapshot's header and exits without
// using a GPU.  Output lines are "%e\t%e\t%d\n": k_eff, P(k), modes, for the
// bins that hold modes (print_pk, utils.cpp:7-21).
//
// Each type is read in chunks of at most 2^26 particles and deposited with
// genpk_deposit (+= across chunks, as read_fieldize.cpp:41-93 calls fieldize);
// the normalising mass is the sum of the particle masses, plus 1 for a Gadget
// snapshot (read_fieldize.cpp:94) and nothing more for a BigFile one
// (read_fieldize_bigfile.cpp:117): the reference's own conventions.
#include "bigfile.h"
#include "gadget2.h"
#include "genpk_gb300.h"

#include <memory>

#include <getopt.h>

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

// Particle types (GadgetReader's numbering, which the reference uses).
constexpr int kBaryon = 0, kDM = 1, kNeutrino = 2, kStars = 4;
constexpr int64_t kFieldDimsMax = 3072;        // FIELD_DIMS, gen-pk.cpp:63
constexpr int64_t kChunk = (int64_t)1 << 26;   // read_fieldize.cpp:41

std::string type_str(int type)
{
    switch (type) {
    case kBaryon:
        return "by";
    case kDM:
        return "DM";
    case kNeutrino:
        return "nu";
    case kStars:
        return "st";
    default:
        return "xx";
    }
}

// Smallest power of two >= n (n >= 1); 0 for n = 0.
int64_t next_pow2(int64_t n)
{
    if (n <= 0)
        return 0;
    int64_t p = 1;
    while (p < n)
        p <<= 1;
    return p;
}

void usage()
{
    fprintf(stderr,
            "Usage: gen-pk-gb300 -i snapshot -o outdir [-j snapshot2] [-c type] [-s 0|1]\n"
            "                    [-g grid] [-b bins] [-d] [-h]\n"
            "Writes one file per particle type, outdir/PK-$TYPE-$INPUT, with three columns per\n"
            "non-empty bin: k_eff, P(k), number of modes.\n"
            "  -j  cross spectrum of each type with the same type in snapshot2 (PX-$TYPE-$INPUT)\n"
            "  -c  cross spectrum of the dark matter (type 1) with this type (PK-DMx$TYPE-$INPUT)\n"
            "  -s  1: add the stars (type 4) to the baryons (type 0)\n"
            "  -g  grid size (default: max over types of min(2*nexttwo(cbrt(npart)), 3072))\n"
            "  -b  number of log-k bins (default: the grid size)\n"
            "  -d  print the snapshot header and exit\n");
}

struct Fail : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// A snapshot in either format, as the driver uses it.
class Source {
public:
    explicit Source(const std::string &path)
    {
        if (bigfile::Snapshot::is_bigfile(path)) {
            bf_.reset(new bigfile::Snapshot(path));
            return;
        }
        FILE *f = fopen(path.c_str(), "rb");
        if (f) {
            unsigned char sig[8] = {};
            const size_t got = fread(sig, 1, 8, f);
            fclose(f);
            static const unsigned char hdf5[8] = {0x89, 'H', 'D', 'F', '\r', '\n', 0x1a, '\n'};
            if (got == 8 && memcmp(sig, hdf5, 8) == 0)
                throw Fail(path + " is an HDF5 snapshot: this build has no HDF5 library");
        }
        g2_.reset(new g2::Snapshot(path));
    }
    const char *format() const { return bf_ ? "bigfile" : "gadget format-II"; }
    int num_files() const { return bf_ ? 1 : g2_->num_files(); }
    int64_t npart(int t) const { return bf_ ? bf_->npart(t) : g2_->npart(t); }
    double mass(int t) const { return bf_ ? bf_->mass(t) : g2_->mass(t); }
    double box() const { return bf_ ? bf_->box() : g2_->box(); }
    double time() const { return bf_ ? bf_->time() : g2_->header().time; }
    double redshift() const { return bf_ ? 1.0 / bf_->time() - 1.0 : g2_->header().redshift; }
    double hubble() const { return bf_ ? bf_->hubble() : g2_->header().hubble; }
    double omega0() const { return bf_ ? bf_->omega0() : g2_->header().omega0; }
    // Added to each type's normalising mass per read: read_fieldize.cpp:94
    // (Gadget) adds 1, read_fieldize_bigfile.cpp:117 (BigFile) nothing.
    double mass_offset() const { return bf_ ? 0.0 : 1.0; }
    void read(int type, int64_t start, int64_t n, float *pos, float *m) const
    {
        if (bf_)
            bf_->read(type, start, n, pos, m);
        else
            g2_->read(type, start, n, pos, m);
    }

private:
    std::unique_ptr<g2::Snapshot> g2_;
    std::unique_ptr<bigfile::Snapshot> bf_;
};

void check(genpk_ctx *ctx, int status, const char *what)
{
    if (status != GENPK_OK)
        throw Fail(std::string(what) + ": " + genpk_status_string(status) +
                   (ctx ? std::string(" (") + genpk_last_error(ctx) + ")" : ""));
}

// Deposit every particle of `type` into grid `field`; adds the normalising
// mass (particle masses + the format's offset) to *total_mass.  Returns false
// if the snapshot holds no particle of that type.
bool read_fieldize(genpk_ctx *ctx, int field, const Source &snap, int type, double *total_mass)
{
    const int64_t n = snap.npart(type);
    if (n == 0)
        return false;
    const double mass = snap.mass(type);
    const int64_t chunk = std::min(n, kChunk);
    std::vector<float> pos((size_t)(3 * chunk));
    std::vector<float> masses(mass == 0.0 ? (size_t)chunk : 0);
    for (int64_t start = 0; start < n; start += chunk) {
        const int64_t parts = std::min(chunk, n - start);
        snap.read(type, start, parts, pos.data(), masses.empty() ? nullptr : masses.data());
        if (mass == 0.0) {
            double s = 0.0;
            for (int64_t i = 0; i < parts; i++)
                s += masses[(size_t)i];
            *total_mass += s;
        }
        *total_mass += mass * (double)parts;
        check(ctx,
              genpk_deposit(ctx, field, snap.box(), pos.data(),
                            masses.empty() ? nullptr : masses.data(), mass, parts),
              "genpk_deposit");
    }
    *total_mass += snap.mass_offset();
    return true;
}

bool print_pk(const std::string &filename, int nrbins, const std::vector<double> &keffs,
              const std::vector<double> &power, const std::vector<int> &count)
{
    FILE *fd = fopen(filename.c_str(), "w");
    if (!fd) {
        fprintf(stderr, "Error opening file: %s\n", filename.c_str());
        return false;
    }
    for (int i = 0; i < nrbins; i++)
        if (count[(size_t)i])
            fprintf(fd, "%e\t%e\t%d\n", keffs[(size_t)i], power[(size_t)i], count[(size_t)i]);
    fclose(fd);
    return true;
}

int run(int argc, char **argv)
{
    std::string infiles, jinfiles, outdir;
    int crosstype = -1;
    bool stars_are_baryons = false, describe = false;
    int64_t grid = 0;
    int bins = 0;
    int c;
    while ((c = getopt(argc, argv, "i:j:o:c:s:g:b:dh")) != -1) {
        switch (c) {
        case 'o':
            outdir = optarg;
            break;
        case 'i':
            infiles = optarg;
            break;
        case 'j':
            jinfiles = optarg;
            break;
        case 'c':
            crosstype = atoi(optarg);
            break;
        case 's':
            stars_are_baryons = atoi(optarg) != 0;
            break;
        case 'g':
            grid = atoll(optarg);
            break;
        case 'b':
            bins = atoi(optarg);
            break;
        case 'd':
            describe = true;
            break;
        case 'h':
        default:
            usage();
            return 0;
        }
    }
    if (infiles.empty() || (outdir.empty() && !describe)) {
        usage();
        return 0;
    }
    const Source snap(infiles);
    int64_t npart[g2::kTypes];
    for (int t = 0; t < g2::kTypes; t++)
        npart[t] = snap.npart(t);
    printf("Boxsize=%g, ", snap.box());
    printf("NPart=(%g,%g,%g,%g,%g,%g)**3\n", cbrt((double)npart[0]), cbrt((double)npart[1]),
           cbrt((double)npart[2]), cbrt((double)npart[3]), cbrt((double)npart[4]),
           cbrt((double)npart[5]));
    printf("Masses=[%g %g %g ]\n", snap.mass(0), snap.mass(1), snap.mass(2));
    printf("redshift=%g, Omega_M=%g\n", snap.redshift(), snap.omega0());
    if (describe) {
        printf("format=%s files=%d time=%g h=%g\n", snap.format(), snap.num_files(), snap.time(),
               snap.hubble());
        for (int t = 0; t < g2::kTypes; t++)
            printf("type %d (%s): npart=%lld mass=%.10g\n", t, type_str(t).c_str(),
                   (long long)npart[t], snap.mass(t));
        return 0;
    }

    int64_t field_dims = 0;
    for (int t = 0; t < g2::kTypes; t++) {
        // the reference converts cbrt's double to int before rounding up
        const int64_t tmp = 2 * next_pow2((int64_t)cbrt((double)npart[t]));
        field_dims = std::max(field_dims, std::min(tmp, kFieldDimsMax));
    }
    if (grid > 0)
        field_dims = grid;
    const int nrbins = bins > 0 ? bins : (int)field_dims;
    printf("FFT grid dimension: %lld\n", (long long)field_dims);

    genpk_ctx *ctx = nullptr;
    check(nullptr, genpk_ctx_create(field_dims, nrbins, 2, 0, &ctx), "genpk_ctx_create");
    struct Guard {
        genpk_ctx *c;
        ~Guard() { genpk_ctx_destroy(c); }
    } guard{ctx};
    std::vector<double> power((size_t)nrbins), keffs((size_t)nrbins);
    std::vector<int> count((size_t)nrbins);
    const size_t last = infiles.find_last_of("/\\");
    const std::string input = infiles.substr(last == std::string::npos ? 0 : last + 1);

    if (crosstype < 0 && jinfiles.empty()) {
        // a spectrum for each particle type (gen-pk.cpp:202-239)
        for (int type = 0; type < g2::kTypes; type++) {
            if (npart[type] == 0)
                continue;
            check(ctx, genpk_zero(ctx, 0), "genpk_zero");
            double total_mass = 0.0;
            read_fieldize(ctx, 0, snap, type, &total_mass);
            if (type == kBaryon && stars_are_baryons)
                read_fieldize(ctx, 0, snap, kStars, &total_mass);
            printf("total_mass in type %d = %g\n", type, total_mass);
            check(ctx, genpk_power(ctx, 0, 0, total_mass, total_mass, power.data(), count.data(),
                                   keffs.data()),
                  "genpk_power");
            print_pk(outdir + "/PK-" + type_str(type) + "-" + input, nrbins, keffs, power, count);
        }
    } else if (!jinfiles.empty()) {
        // each type against the same type of a second snapshot (gen-pk.cpp:240-303)
        const Source snap2(jinfiles);
        for (int type = 0; type < g2::kTypes; type++) {
            if (npart[type] == 0)
                continue;
            check(ctx, genpk_zero(ctx, 0), "genpk_zero");
            check(ctx, genpk_zero(ctx, 1), "genpk_zero");
            double m1 = 0.0, m2 = 0.0;
            if (!read_fieldize(ctx, 0, snap, type, &m1) || !read_fieldize(ctx, 1, snap2, type, &m2))
                continue;
            check(ctx, genpk_power(ctx, 0, 1, m1, m2, power.data(), count.data(), keffs.data()),
                  "genpk_power");
            print_pk(outdir + "/PX-" + type_str(type) + "-" + input, nrbins, keffs, power, count);
        }
    } else {
        // the dark matter against one other type (gen-pk.cpp:304-356)
        if (crosstype >= g2::kTypes || npart[kDM] == 0 || npart[crosstype] == 0) {
            fprintf(stderr, "Can't cross-correlate types not present in snapshot\n");
            return 1;
        }
        check(ctx, genpk_zero(ctx, 0), "genpk_zero");
        check(ctx, genpk_zero(ctx, 1), "genpk_zero");
        double m1 = 0.0, m2 = 0.0;
        read_fieldize(ctx, 0, snap, kDM, &m1);
        read_fieldize(ctx, 1, snap, crosstype, &m2);
        check(ctx, genpk_power(ctx, 0, 1, m1, m2, power.data(), count.data(), keffs.data()),
              "genpk_power");
        print_pk(outdir + "/PK-DMx" + type_str(crosstype) + "-" + input, nrbins, keffs, power,
                 count);
    }
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    try {
        return run(argc, argv);
    } catch (const std::exception &e) {
        fprintf(stderr, "gen-pk-gb300: %s\n", e.what());
        return 1;
    }
}
