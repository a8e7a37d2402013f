// compat.cpp -- libgenpk_compat.so: the reference's fieldize / invwindow /
// powerspectrum signatures (gen-pk.h:93,104,119) on top of the C ABI.
#include <string.h>

#include <map>
#include <mutex>
#include <utility>
#include <vector>

#include "../../include/genpk_compat.h"

namespace {

struct Binding {
    genpk_ctx *ctx;
    int field;
};

std::mutex g_mu;
std::map<const void *, Binding> g_bind;
std::map<std::pair<int64_t, int>, genpk_ctx *> g_private;  // (dims, nrbins) -> ctx

genpk_ctx *private_ctx(int64_t dims, int nrbins)
{
    auto key = std::make_pair(dims, nrbins);
    auto it = g_private.find(key);
    if (it != g_private.end())
        return it->second;
    genpk_ctx *ctx = nullptr;
    if (genpk_ctx_create(dims, nrbins, 2, 0, &ctx) != GENPK_OK) {
        genpk_ctx_destroy(ctx);
        return nullptr;
    }
    g_private[key] = ctx;
    return ctx;
}

const Binding *find_binding(const void *p)
{
    auto it = g_bind.find(p);
    return it == g_bind.end() ? nullptr : &it->second;
}

}  // namespace

int fieldize(double boxsize, int dims, double *out, int64_t segment_particles, float *positions,
             float *masses, double mass, int extra)
{
    std::lock_guard<std::mutex> lock(g_mu);
    if (const Binding *b = find_binding(out)) {
        if (extra != 1)
            return GENPK_ERR_UNSUPPORTED;
        int rc = genpk_deposit(b->ctx, b->field, boxsize, positions, masses, mass,
                               segment_particles);
        if (rc == GENPK_ERR_STATE) {
            // The grid still holds the previous species' spectrum: the driver
            // memsets its host field before the next species (gen-pk.cpp:208),
            // which never reaches the device, so start the grid afresh here.
            rc = genpk_zero(b->ctx, b->field);
            if (rc == GENPK_OK)
                rc = genpk_deposit(b->ctx, b->field, boxsize, positions, masses, mass,
                                   segment_particles);
        }
        return rc;
    }
    if (!out || dims < 2 || (extra != 0 && extra != 1) || (extra == 0 && (dims & 1)))
        return GENPK_ERR_INVALID;
    genpk_ctx *ctx = private_ctx(dims, 1);
    if (!ctx)
        return GENPK_ERR_CUDA;
    int rc = genpk_zero(ctx, 0);
    if (rc == GENPK_OK)
        rc = genpk_deposit(ctx, 0, boxsize, positions, masses, mass, segment_particles);
    const size_t row = 2 * (size_t)(dims / 2 + 1);
    std::vector<double> g((size_t)dims * dims * row);
    if (rc == GENPK_OK)
        rc = genpk_read_field(ctx, 0, g.data());
    if (rc != GENPK_OK)
        return rc;
    // fieldize.cpp:48-51: rows of fdims = 2*(dims/2 + extra) doubles.
    const size_t fdims = 2 * (size_t)(dims / 2 + extra);
    for (int x = 0; x < dims; x++)
        for (int y = 0; y < dims; y++)
            for (int z = 0; z < dims; z++)
                out[((size_t)x * dims + y) * fdims + z] += g[((size_t)x * dims + y) * row + z];
    return GENPK_OK;
}

extern "C" {

double invwindow(int64_t kx, int64_t ky, int64_t kz, int64_t n)
{
    return genpk_invwindow(kx, ky, kz, n);
}

int powerspectrum(int64_t dims, double (*outfield)[2], double (*outfield2)[2], int nrbins,
                  double *power, int *count, double *keffs, double total_mass, double total_mass2)
{
    std::lock_guard<std::mutex> lock(g_mu);
    const Binding *a = find_binding(outfield);
    const Binding *b = find_binding(outfield2);
    if (a && b) {
        if (a->ctx != b->ctx)
            return GENPK_ERR_INVALID;
        return genpk_power(a->ctx, a->field, b->field, total_mass, total_mass2, power, count, keffs);
    }
    if (!outfield || !outfield2 || dims < 2 || nrbins < 1)
        return GENPK_ERR_INVALID;
    genpk_ctx *ctx = private_ctx(dims, nrbins);
    if (!ctx)
        return GENPK_ERR_CUDA;
    int rc = genpk_load_spectrum(ctx, 0, &outfield[0][0]);
    int fb = 0;
    if (rc == GENPK_OK && outfield2 != outfield) {
        rc = genpk_load_spectrum(ctx, 1, &outfield2[0][0]);
        fb = 1;
    }
    if (rc != GENPK_OK)
        return rc;
    return genpk_power(ctx, 0, fb, total_mass, total_mass2, power, count, keffs);
}

int genpk_compat_bind(genpk_ctx *ctx, int field, const void *host_field)
{
    if (!ctx || !host_field)
        return GENPK_ERR_INVALID;
    std::lock_guard<std::mutex> lock(g_mu);
    g_bind[host_field] = Binding{ctx, field};
    return genpk_zero(ctx, field);
}

int genpk_compat_unbind(const void *host_field)
{
    std::lock_guard<std::mutex> lock(g_mu);
    return g_bind.erase(host_field) ? GENPK_OK : GENPK_ERR_INVALID;
}

void genpk_compat_release(void)
{
    std::lock_guard<std::mutex> lock(g_mu);
    for (auto &kv : g_private)
        genpk_ctx_destroy(kv.second);
    g_private.clear();
}

}  // extern "C"
