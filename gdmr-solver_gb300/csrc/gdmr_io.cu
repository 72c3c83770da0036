// On-disk deflation spaces (gdmr_deflation_* in gdmr_ext.h).
//
// The reference can only move its source-side deflation vectors between host and device
// (impSVDMR/expSVDMR, gDMR.cu:431-477), so a recycled space dies with the process.  This
// file gives it a versioned file format, so a later process (or another machine) can start
// from it with mode != 0:
//
//   offset  size  field
//        0     8  magic "GDMRDEFL"
//        8     4  format version (1), little endian
//       12     4  k (vectors)
//       16     8  n (vector length)
//       24     8  FNV-1a 64-bit hash of the payload bytes
//       32  16kn  payload: k vectors of n complex128 values (re, im), vector-contiguous
//
// All integers little endian; the payload is IEEE-754 binary64.  Reading checks the magic,
// the version, the sizes against the caller's and the hash.
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "gdmr_engine.h"

extern "C" {
#include "../../include/gdmr_ext.h"
}

using namespace gdmr;

namespace {

constexpr char kMagic[8] = {'G', 'D', 'M', 'R', 'D', 'E', 'F', 'L'};
constexpr uint32_t kVersion = 1;

uint64_t fnv1a(const unsigned char *p, size_t len) {
    uint64_t h = 1469598103934665603ull;
    for (size_t i = 0; i < len; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

void put32(unsigned char *d, uint32_t v) {
    for (int i = 0; i < 4; ++i) d[i] = (unsigned char)(v >> (8 * i));
}
void put64(unsigned char *d, uint64_t v) {
    for (int i = 0; i < 8; ++i) d[i] = (unsigned char)(v >> (8 * i));
}
uint32_t get32(const unsigned char *d) {
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i) v |= (uint32_t)d[i] << (8 * i);
    return v;
}
uint64_t get64(const unsigned char *d) {
    uint64_t v = 0;
    for (int i = 0; i < 8; ++i) v |= (uint64_t)d[i] << (8 * i);
    return v;
}

// Payload as little-endian bytes regardless of the host's byte order.
std::vector<unsigned char> to_bytes(const double *z, size_t count) {
    std::vector<unsigned char> out(count * 8);
    for (size_t i = 0; i < count; ++i) {
        uint64_t bits;
        std::memcpy(&bits, &z[i], 8);
        put64(&out[i * 8], bits);
    }
    return out;
}

int io_fail(int status, const std::string &msg) {
    set_last_error(status, msg);
    return status;
}

}  // namespace

extern "C" int gdmr_deflation_write(const char *path, int n, int k, const double *z) {
    if (!path || !z || n <= 0 || k <= 0) return io_fail(GDMR_EINVAL, "gdmr_deflation_write: bad argument");
    const size_t count = (size_t)2 * n * k;
    std::vector<unsigned char> payload = to_bytes(z, count);
    unsigned char hdr[32];
    std::memcpy(hdr, kMagic, 8);
    put32(hdr + 8, kVersion);
    put32(hdr + 12, (uint32_t)k);
    put64(hdr + 16, (uint64_t)n);
    put64(hdr + 24, fnv1a(payload.data(), payload.size()));
    const std::string tmp = std::string(path) + ".tmp";
    FILE *f = fopen(tmp.c_str(), "wb");
    if (!f) return io_fail(GDMR_EINVAL, std::string("gdmr_deflation_write: cannot open ") + tmp);
    bool ok = fwrite(hdr, 1, 32, f) == 32 && fwrite(payload.data(), 1, payload.size(), f) == payload.size();
    ok = (fclose(f) == 0) && ok;
    if (!ok || std::rename(tmp.c_str(), path) != 0) {
        std::remove(tmp.c_str());
        return io_fail(GDMR_EINVAL, std::string("gdmr_deflation_write: write failed for ") + path);
    }
    set_last_error(GDMR_OK, "ok");
    return GDMR_OK;
}

extern "C" int gdmr_deflation_read(const char *path, int n, int k, double *z) {
    if (!path || !z || n <= 0 || k <= 0) return io_fail(GDMR_EINVAL, "gdmr_deflation_read: bad argument");
    FILE *f = fopen(path, "rb");
    if (!f) return io_fail(GDMR_EINVAL, std::string("gdmr_deflation_read: cannot open ") + path);
    unsigned char hdr[32];
    if (fread(hdr, 1, 32, f) != 32) {
        fclose(f);
        return io_fail(GDMR_EINVAL, "gdmr_deflation_read: truncated header");
    }
    if (std::memcmp(hdr, kMagic, 8) != 0) {
        fclose(f);
        return io_fail(GDMR_EINVAL, "gdmr_deflation_read: not a deflation-space file");
    }
    if (get32(hdr + 8) != kVersion) {
        fclose(f);
        return io_fail(GDMR_EINVAL, "gdmr_deflation_read: unsupported format version");
    }
    if (get32(hdr + 12) != (uint32_t)k || get64(hdr + 16) != (uint64_t)n) {
        fclose(f);
        return io_fail(GDMR_EINVAL, "gdmr_deflation_read: file holds a different k or n");
    }
    const size_t count = (size_t)2 * n * k;
    std::vector<unsigned char> payload(count * 8);
    const size_t got = fread(payload.data(), 1, payload.size(), f);
    fclose(f);
    if (got != payload.size()) return io_fail(GDMR_EINVAL, "gdmr_deflation_read: truncated payload");
    if (fnv1a(payload.data(), payload.size()) != get64(hdr + 24))
        return io_fail(GDMR_EINVAL, "gdmr_deflation_read: checksum mismatch");
    for (size_t i = 0; i < count; ++i) {
        const uint64_t bits = get64(&payload[i * 8]);
        std::memcpy(&z[i], &bits, 8);
    }
    set_last_error(GDMR_OK, "ok");
    return GDMR_OK;
}
