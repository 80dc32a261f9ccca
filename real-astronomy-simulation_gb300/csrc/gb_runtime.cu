// Host runtime shared by every entry point: error reporting and device info.
#include <cmath>
#include <cstdarg>
#include <cstdio>

#include "gb_common.cuh"

namespace gb {

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int fail(int code, const char *fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int make_extpot(const gb_potential_t *pot, float G, ExtPot *out) {
    *out = ExtPot{};
    if (!pot) return GB_OK;
    const double v[] = {pot->M_d, pot->a, pot->b, pot->M_h, pot->a_h, pot->smbh_mass};
    for (double x : v)
        if (!std::isfinite(x)) return fail(GB_EINVAL, "potential parameters must be finite");
    if (pot->reserved != 0) return fail(GB_EINVAL, "gb_potential_t.reserved must be 0");
    if (pot->is_hernquist != 0 && pot->is_hernquist != 1)
        return fail(GB_EINVAL, "is_hernquist must be 0 or 1 (got %d)", (int)pot->is_hernquist);
    out->gmd = (float)((double)G * pot->M_d);
    out->a = (float)pot->a;
    out->b = (float)pot->b;
    out->gmh = (float)((double)G * pot->M_h);
    out->ah = (float)pot->a_h;
    out->gmbh = (float)((double)G * pot->smbh_mass);
    out->hernquist = pot->is_hernquist;
    out->smbh = pot->smbh_mass > 0.0 ? 1 : 0;
    out->on = 1;
    return GB_OK;
}

int num_sms() {
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return 1;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
    return sms > 0 ? sms : 1;
}

int read_diag(unsigned long long *dev, gb_diag_t *out, int reset) {
    unsigned long long d[DIAG_COUNT];
    GB_CUDA_TRY(cudaMemcpy(d, dev, sizeof(d), cudaMemcpyDeviceToHost));
    out->stack_drops = d[DIAG_STACK_DROPS];
    out->stack_overflow = d[DIAG_STACK_OVERFLOW];
    out->nonfinite = d[DIAG_NONFINITE];
    out->bad_tree = d[DIAG_BAD_TREE];
    out->warp_node_reads = d[DIAG_NODE_READS];
    out->warp_root_reads = d[DIAG_ROOT_READS];
    out->lane_interactions = d[DIAG_INTERACTIONS];
    out->lane_tests = d[DIAG_TESTS];
    out->wait_timeouts = d[DIAG_WAIT_TIMEOUT];
    if (reset) GB_CUDA_TRY(cudaMemset(dev, 0, sizeof(d)));
    return GB_OK;
}

}  // namespace gb

extern "C" const char *gb_last_error_string(void) { return gb::g_err; }

extern "C" int gb_version(void) { return 10000; }
