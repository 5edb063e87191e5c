// io.cu -- the reference's checkpoint files: Fortran unformatted sequential
// records as GRAVA writes them (solver/gravar_incomp.f90:19-51) and
// leer_campos reads them (solver/leer_incomp.f90:45-116).  Host code.
//
// A record is a 4-byte length marker, the data, the same marker again
// (integers 4 bytes, reals 8 bytes: ifort -r8, solver/mix3d.mk:2-3).  Records
// of 2^31 bytes or more are split into subrecords whose markers carry a sign:
// a negative leading marker means more subrecords follow, a negative trailing
// marker means subrecords preceded this one (the gfortran convention).
//
//   field_SS.NNN    nd | nx ny nz | u | v | w | temp | pres
//   time_SS.NNN     dto it
//   impellermask_SS.NNN   mask
//   sobject.field   nx ny nz | sobject
#include "common.cuh"

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <vector>

namespace emix {
namespace {

constexpr int64_t kMaxSub = 2147483639;   // largest subrecord payload (2^31 - 9)

struct File {
    FILE *fp = nullptr;
    explicit File(const char *path, const char *mode) { fp = std::fopen(path, mode); }
    ~File() {
        if (fp) std::fclose(fp);
    }
};

bool put_marker(FILE *fp, int32_t m) { return std::fwrite(&m, 4, 1, fp) == 1; }

bool write_record(FILE *fp, const void *data, int64_t bytes) {
    const unsigned char *p = static_cast<const unsigned char *>(data);
    int64_t left = bytes;
    bool first = true;
    do {
        const int64_t chunk = left > kMaxSub ? kMaxSub : left;
        const bool more = left > chunk;
        const int32_t lead = more ? -(int32_t)chunk : (int32_t)chunk;
        const int32_t tail = first ? (int32_t)chunk : -(int32_t)chunk;
        if (!put_marker(fp, lead)) return false;
        if (chunk && std::fwrite(p, 1, (size_t)chunk, fp) != (size_t)chunk) return false;
        if (!put_marker(fp, tail)) return false;
        p += chunk;
        left -= chunk;
        first = false;
    } while (left > 0);
    return true;
}

// reads one record into out (exactly `bytes` expected); returns false on a
// size mismatch or a short file
bool read_record(FILE *fp, void *out, int64_t bytes) {
    unsigned char *p = static_cast<unsigned char *>(out);
    int64_t got = 0;
    for (;;) {
        int32_t lead, tail;
        if (std::fread(&lead, 4, 1, fp) != 1) return false;
        const int64_t chunk = lead < 0 ? -(int64_t)lead : lead;
        if (got + chunk > bytes) return false;
        if (chunk && std::fread(p + got, 1, (size_t)chunk, fp) != (size_t)chunk) return false;
        if (std::fread(&tail, 4, 1, fp) != 1) return false;
        if ((tail < 0 ? -(int64_t)tail : tail) != chunk) return false;
        got += chunk;
        if (lead >= 0) break;
    }
    return got == bytes;
}

int io_fail(const char *what, const char *path) {
    char buf[512];
    std::snprintf(buf, sizeof buf, "%s: %s", what, path ? path : "(null)");
    set_last_message(buf);
    return EMIX_ERR_ARG;
}

} // namespace
} // namespace emix

using namespace emix;

extern "C" {

int emix_write_field(const char *path, int nd, int nx, int ny, int nz, const double *u,
                     const double *temp, const double *pres) {
    if (!path || !u || !temp || !pres || nx < 1 || ny < 1 || nz < 1) return EMIX_ERR_ARG;
    File f(path, "wb");
    if (!f.fp) return io_fail("cannot open for writing", path);
    const int64_t n = (int64_t)nx * ny * nz, b = n * 8;
    const int32_t dims[3] = {nx, ny, nz};
    const int32_t nd4 = nd;
    bool ok = write_record(f.fp, &nd4, 4) && write_record(f.fp, dims, 12);
    for (int c = 0; c < 3 && ok; ++c) ok = write_record(f.fp, u + c * n, b);
    ok = ok && write_record(f.fp, temp, b) && write_record(f.fp, pres, b);
    return ok ? EMIX_OK : io_fail("write failed", path);
}

int emix_read_field(const char *path, int nd, int nx, int ny, int nz, double *u, double *temp,
                    double *pres) {
    if (!path || !u || !temp || !pres || nx < 1 || ny < 1 || nz < 1) return EMIX_ERR_ARG;
    File f(path, "rb");
    if (!f.fp) return io_fail("cannot open for reading", path);
    int32_t nd4 = 0, dims[3] = {0, 0, 0};
    // the checks of leer_incomp.f90:68-74
    if (!read_record(f.fp, &nd4, 4) || nd4 != nd) return io_fail("number of variables differs", path);
    if (!read_record(f.fp, dims, 12) || dims[0] != nx || dims[1] != ny || dims[2] != nz)
        return io_fail("dimensions differ", path);
    const int64_t n = (int64_t)nx * ny * nz, b = n * 8;
    bool ok = true;
    for (int c = 0; c < 3 && ok; ++c) ok = read_record(f.fp, u + c * n, b);
    ok = ok && read_record(f.fp, temp, b) && read_record(f.fp, pres, b);
    return ok ? EMIX_OK : io_fail("field records unreadable", path);
}

int emix_write_time(const char *path, double dto, int it) {
    if (!path) return EMIX_ERR_ARG;
    File f(path, "wb");
    if (!f.fp) return io_fail("cannot open for writing", path);
    unsigned char rec[12];
    const int32_t it4 = it;
    std::memcpy(rec, &dto, 8);
    std::memcpy(rec + 8, &it4, 4);
    return write_record(f.fp, rec, 12) ? EMIX_OK : io_fail("write failed", path);
}

int emix_read_time(const char *path, double *dto, int *it) {
    if (!path || !dto || !it) return EMIX_ERR_ARG;
    File f(path, "rb");
    if (!f.fp) return io_fail("cannot open for reading", path);
    unsigned char rec[12];
    if (!read_record(f.fp, rec, 12)) return io_fail("time record unreadable", path);
    int32_t it4;
    std::memcpy(dto, rec, 8);
    std::memcpy(&it4, rec + 8, 4);
    *it = it4;
    return EMIX_OK;
}

int emix_write_array(const char *path, const double *a, long n) {
    if (!path || !a || n < 0) return EMIX_ERR_ARG;
    File f(path, "wb");
    if (!f.fp) return io_fail("cannot open for writing", path);
    return write_record(f.fp, a, (int64_t)n * 8) ? EMIX_OK : io_fail("write failed", path);
}

int emix_read_array(const char *path, double *a, long n) {
    if (!path || !a || n < 0) return EMIX_ERR_ARG;
    File f(path, "rb");
    if (!f.fp) return io_fail("cannot open for reading", path);
    return read_record(f.fp, a, (int64_t)n * 8) ? EMIX_OK : io_fail("array record unreadable", path);
}

int emix_read_sobject(const char *path, int nx, int ny, int nz, double *sobject) {
    if (!path || !sobject || nx < 1 || ny < 1 || nz < 1) return EMIX_ERR_ARG;
    File f(path, "rb");
    if (!f.fp) return io_fail("cannot open for reading", path);
    int32_t dims[3];
    if (!read_record(f.fp, dims, 12) || dims[0] != nx || dims[1] != ny || dims[2] != nz)
        return io_fail("dimensions differ", path);
    return read_record(f.fp, sobject, (int64_t)nx * ny * nz * 8) ? EMIX_OK
                                                                   : io_fail("sobject unreadable", path);
}

} // extern "C"
