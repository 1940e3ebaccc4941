// Plan cache: the GPU counterpart of FFTW wisdom (fft_init's third argument,
// src/fft.c:26-45).  FFTW_MEASURE times FFT algorithms and the wisdom file
// keeps the winners; here the tunables are the launch shapes of the three
// FP32 r2c passes (fft2.cu: k-pass rows per CTA, j- and i-pass columns per
// CTA), measured by fft2_autotune on the device and kept in a text file with
// one line per (compute capability, SM count, Ng, precision):
//
//   fftgal_gb300-plan 1 cc=103 sms=152 Ng=1024 prec=4 kR=4 jlogC=3 ilogC=4 ms=4.010,4.290,4.660 dev=<name>
//
// and, for FP32 grids, the launch shapes of the tile paint (persistent CTAs
// per SM) and of the finish + binning kernel (CTAs per SM, blocks between
// the folds of its FP32 sums) on lines of their own (launch_store).
//
// Other lines of the file are kept as they are.  Entries measured in this
// process are also kept in memory, so a second grid of the same size is not
// measured again.
#include "internal.h"
#include "fftgal_gb300.h"

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>
#include <chrono>
#include <unistd.h>

namespace fg {

static double wall_seconds() {
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

static const char kTag[] = "fftgal_gb300-plan 1 ";

static bool parse_line(const char *line, int *cc, int *sms, int *Ng, int *prec, int tun[3]) {
    if (strncmp(line, kTag, sizeof(kTag) - 1)) return false;
    int c, s, n, p, a, b, d;
    if (sscanf(line + sizeof(kTag) - 1, "cc=%d sms=%d Ng=%d prec=%d kR=%d jlogC=%d ilogC=%d", &c, &s, &n, &p, &a, &b,
               &d) != 7)
        return false;
    *cc = c;
    *sms = s;
    *Ng = n;
    *prec = p;
    tun[0] = a;
    tun[1] = b;
    tun[2] = d;
    return true;
}

static bool read_lines(const char *path, std::vector<std::string> *lines) {
    FILE *fp = fopen(path, "r");
    if (!fp) return false;
    std::string cur;
    int ch;
    while ((ch = fgetc(fp)) != EOF) {
        if (ch == '\n') {
            lines->push_back(cur);
            cur.clear();
        } else {
            cur.push_back((char)ch);
        }
    }
    if (!cur.empty()) lines->push_back(cur);
    fclose(fp);
    return true;
}

int plan_lookup(const char *path, int cc, int sms, int Ng, int prec, int tun[3]) {
    std::vector<std::string> lines;
    if (!read_lines(path, &lines)) return 0;
    int found = 0;
    for (const auto &l : lines) {  // the last matching line wins
        int c, s, n, p, t[3];
        if (parse_line(l.c_str(), &c, &s, &n, &p, t) && c == cc && s == sms && n == Ng && p == prec) {
            tun[0] = t[0];
            tun[1] = t[1];
            tun[2] = t[2];
            found = 1;
        }
    }
    return found;
}

// the file with every line for which `same` holds replaced by `line`
template <typename F>
static int replace_line(const char *path, F same, const char *line) {
    std::vector<std::string> lines, keep;
    read_lines(path, &lines);
    for (const auto &l : lines)
        if (!same(l.c_str())) keep.push_back(l);
    keep.push_back(line);
    // write beside the target and rename, so a reader never sees half a file
    std::string tmp = std::string(path) + ".tmp" + std::to_string((long)getpid());
    FILE *fp = fopen(tmp.c_str(), "w");
    if (!fp) return set_error(ERR_IO, "cannot write plan file %s", tmp.c_str());
    bool ok = true;
    for (const auto &l : keep) ok = ok && fprintf(fp, "%s\n", l.c_str()) > 0;
    ok = (fclose(fp) == 0) && ok;
    if (!ok || rename(tmp.c_str(), path) != 0) {
        remove(tmp.c_str());
        return set_error(ERR_IO, "cannot write plan file %s", path);
    }
    return OK;
}

int plan_store(const char *path, int cc, int sms, int Ng, int prec, const int tun[3], const double ms[3],
               const char *dev) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%scc=%d sms=%d Ng=%d prec=%d kR=%d jlogC=%d ilogC=%d ms=%.3f,%.3f,%.3f dev=%s", kTag,
             cc, sms, Ng, prec, tun[0], tun[1], tun[2], ms ? ms[0] : 0.0, ms ? ms[1] : 0.0, ms ? ms[2] : 0.0,
             dev ? dev : "");
    return replace_line(path, [&](const char *l) {
        int c, s, n, p, t[3];
        return parse_line(l, &c, &s, &n, &p, t) && c == cc && s == sms && n == Ng && p == prec;
    }, buf);
}

// ---- launch shapes of the paint and binning kernels ------------------------------------------
//   fftgal_gb300-launch 1 cc=103 sms=152 Ng=1024 paint_cta=2 bin_cta=3 bin_fold=8 ms=11.8,5.1 dev=<name>
static const char kLTag[] = "fftgal_gb300-launch 1 ";

static bool parse_launch(const char *line, int *cc, int *sms, int *Ng, LaunchTune *t) {
    if (strncmp(line, kLTag, sizeof(kLTag) - 1)) return false;
    int c, s, n, a, b, f;
    if (sscanf(line + sizeof(kLTag) - 1, "cc=%d sms=%d Ng=%d paint_cta=%d bin_cta=%d bin_fold=%d", &c, &s, &n, &a,
               &b, &f) != 6)
        return false;
    *cc = c;
    *sms = s;
    *Ng = n;
    t->paint_cta = a;
    t->bin_cta = b;
    t->bin_fold = f;
    return true;
}

int launch_lookup(const char *path, int cc, int sms, int Ng, LaunchTune *t) {
    std::vector<std::string> lines;
    if (!read_lines(path, &lines)) return 0;
    int found = 0;
    for (const auto &l : lines) {  // the last matching line wins
        int c, s, n;
        LaunchTune u;
        if (parse_launch(l.c_str(), &c, &s, &n, &u) && c == cc && s == sms && n == Ng) {
            *t = u;
            found = 1;
        }
    }
    return found;
}

int launch_store(const char *path, int cc, int sms, int Ng, const LaunchTune &t, const double ms[2], const char *dev) {
    char buf[512];
    snprintf(buf, sizeof(buf), "%scc=%d sms=%d Ng=%d paint_cta=%d bin_cta=%d bin_fold=%d ms=%.3f,%.3f dev=%s", kLTag, cc,
             sms, Ng, t.paint_cta, t.bin_cta, t.bin_fold, ms ? ms[0] : 0.0, ms ? ms[1] : 0.0, dev ? dev : "");
    return replace_line(path, [&](const char *l) {
        int c, s, n;
        LaunchTune u;
        return parse_launch(l, &c, &s, &n, &u) && c == cc && s == sms && n == Ng;
    }, buf);
}

struct DevKey {
    int cc = 0, sms = 0;
    char name[256] = {};
};

static int device_key(DevKey *k) {
    int dev = 0;
    FG_CUDA(cudaGetDevice(&dev));
    cudaDeviceProp prop;
    FG_CUDA(cudaGetDeviceProperties(&prop, dev));
    k->cc = prop.major * 10 + prop.minor;
    k->sms = prop.multiProcessorCount;
    snprintf(k->name, sizeof(k->name), "%s", prop.name);
    return OK;
}

int plan_device_key(int *cc, int *sms, char *name, size_t len) {
    DevKey k;
    FG_TRY(device_key(&k));
    *cc = k.cc;
    *sms = k.sms;
    if (name && len) snprintf(name, len, "%s", k.name);
    return OK;
}

static std::mutex g_cache_mu;
static std::map<std::tuple<int, int, int, int>, std::tuple<int, int, int>> g_cache;

static bool shapes_valid(int Ng, const int tun[3]) {
    for (int w = 0; w < 3; ++w)
        if (!fft2_valid_shape(Ng, w, tun[w])) return false;
    return true;
}

int plan_resolve(FftPlan *p, void *grid, cudaStream_t s, const char *path, bool quiet, int *source, double ms[3]) {
    *source = FFTGAL_PLAN_BUILTIN;
    ms[0] = ms[1] = ms[2] = 0;
    if (!fft2_supported(p->Ng, p->prec)) {
        if (!quiet)
            fprintf(stderr, "fft_init() no tunable launch shapes for Ng=%d (%s grid): built-in GPU plans\n", p->Ng,
                    p->prec == 4 ? "FP32" : "FP64");
        return OK;
    }
    DevKey k;
    FG_TRY(device_key(&k));
    int tun[3];
    if (plan_lookup(path, k.cc, k.sms, p->Ng, p->prec, tun)) {
        if (shapes_valid(p->Ng, tun)) {
            for (int w = 0; w < 3; ++w) p->tune[w] = tun[w];
            *source = FFTGAL_PLAN_FILE;
            if (!quiet) fprintf(stderr, "fft_init() imported plan from %s\n", path);
            std::lock_guard<std::mutex> lk(g_cache_mu);
            g_cache[{k.cc, k.sms, p->Ng, p->prec}] = {tun[0], tun[1], tun[2]};
            return OK;
        }
        if (!quiet) fprintf(stderr, "fft_init() plan for Ng=%d in %s does not fit this device: measuring\n", p->Ng, path);
    }
    bool cached = false;
    {
        std::lock_guard<std::mutex> lk(g_cache_mu);
        auto it = g_cache.find({k.cc, k.sms, p->Ng, p->prec});
        if (it != g_cache.end()) {
            tun[0] = std::get<0>(it->second);
            tun[1] = std::get<1>(it->second);
            tun[2] = std::get<2>(it->second);
            cached = true;
        }
    }
    if (cached) {
        for (int w = 0; w < 3; ++w) p->tune[w] = tun[w];
        *source = FFTGAL_PLAN_CACHE;
    } else {
        const double t0 = wall_seconds();
        FG_TRY(fft2_autotune(p, grid, s, ms));
        for (int w = 0; w < 3; ++w) tun[w] = p->tune[w];
        *source = FFTGAL_PLAN_MEASURED;
        if (!quiet) fprintf(stderr, "fft_init() %.2fs on autotune\n", wall_seconds() - t0);
        std::lock_guard<std::mutex> lk(g_cache_mu);
        g_cache[{k.cc, k.sms, p->Ng, p->prec}] = {tun[0], tun[1], tun[2]};
    }
    // a plan file that cannot be written costs the next run a measurement,
    // not this run its grid: warn and go on with the shapes just found
    if (plan_store(path, k.cc, k.sms, p->Ng, p->prec, tun, ms, k.name) != OK)
        fprintf(stderr, "fft_init() could not export the plan to %s: %s\n", path, fftgal_last_error());
    else if (!quiet)
        fprintf(stderr, "fft_init() exported plan to %s\n", path);
    return OK;
}

}  // namespace fg

using namespace fg;

extern "C" int fftgal_plan_lookup(const char *path, int cc, int sms, int Ng, int prec, int tune[3]) {
    if (!path || !tune) return set_error(ERR_ARG, "fftgal_plan_lookup: null argument");
    return plan_lookup(path, cc, sms, Ng, prec, tune);
}

extern "C" int fftgal_plan_store(const char *path, int cc, int sms, int Ng, int prec, const int tune[3],
                                 const double ms[3], const char *device_name) {
    if (!path || !tune) return set_error(ERR_ARG, "fftgal_plan_store: null argument");
    return plan_store(path, cc, sms, Ng, prec, tune, ms, device_name);
}

extern "C" int fftgal_plan_valid(int Ng, int pass, int shape) {
    if (pass < 0 || pass > 2) return 0;
    return fft2_valid_shape(Ng, pass, shape) ? 1 : 0;
}
