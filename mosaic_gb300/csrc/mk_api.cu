// Library-level entry points: version, error reporting, device status.
#include <stdarg.h>
#include <string.h>

#include <mutex>

#include "mk_common.cuh"

static thread_local char g_err[1024] = "";

void mk_set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

static std::mutex g_readers_mu;
static mk_status_reader g_readers[8];
static int g_n_readers = 0;

void mk_register_status_reader(mk_status_reader fn)
{
    std::lock_guard<std::mutex> lk(g_readers_mu);
    for (int i = 0; i < g_n_readers; ++i)
        if (g_readers[i] == fn) return;
    if (g_n_readers < 8) g_readers[g_n_readers++] = fn;
}

extern "C" int mk_version(void) { return 10000; /* 1.0.0 */ }

extern "C" const char *mk_last_error(void) { return g_err; }

extern "C" int mk_sync_status(void *stream)
{
    cudaStream_t s = mk_stream(stream);
    MK_CHECK_CUDA(cudaStreamSynchronize(s));
    MK_CHECK_CUDA(cudaGetLastError());
    int n;
    mk_status_reader rd[8];
    {
        std::lock_guard<std::mutex> lk(g_readers_mu);
        n = g_n_readers;
        memcpy(rd, g_readers, sizeof(rd));
    }
    int worst = MK_OK;
    for (int i = 0; i < n; ++i) {
        const int st = rd[i](s);
        if (st != MK_OK && worst == MK_OK) worst = st;
    }
    return worst;
}
