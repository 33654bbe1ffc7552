// Gadget-2 snapshots (the reference's SnapFormat 2), host side.
//
// Layout (src/snapshot.c:5-22): a 256-byte header block, a block of FP32
// positions and a block of FP32 velocities, each framed by 4-byte record
// markers, particles in species order 0..5.  Reading converts to FP64 and
// multiplies velocities by (1/(1+z))^1.5 (src/snapshot.c:163-181); writing
// divides by it (src/snapshot.c:470-481).  The header is decoded at fixed
// byte offsets, not by overlaying a struct.
#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "api_internal.cuh"

namespace {

// byte offsets inside the 256-byte header
enum {
    H_NPART = 0, H_MASS = 24, H_TIME = 72, H_REDSHIFT = 80, H_SFR = 88, H_FEEDBACK = 92, H_NTOTAL = 96,
    H_COOLING = 120, H_NFILES = 124, H_BOX = 128, H_OM = 136, H_OL = 144, H_H = 152, H_BYTES = 256
};

template <class T>
T get(const unsigned char *b, int off)
{
    T v;
    memcpy(&v, b + off, sizeof v);
    return v;
}

template <class T>
void put(unsigned char *b, int off, T v)
{
    memcpy(b + off, &v, sizeof v);
}

void decode(const unsigned char *b, photons_gadget_header *h)
{
    for (int i = 0; i < 6; i++) {
        h->npart[i] = get<int>(b, H_NPART + 4 * i);
        h->mass[i] = get<double>(b, H_MASS + 8 * i);
        h->npart_total[i] = get<int>(b, H_NTOTAL + 4 * i);
    }
    h->time = get<double>(b, H_TIME);
    h->redshift = get<double>(b, H_REDSHIFT);
    h->flag_sfr = get<int>(b, H_SFR);
    h->flag_feedback = get<int>(b, H_FEEDBACK);
    h->flag_cooling = get<int>(b, H_COOLING);
    h->num_files = get<int>(b, H_NFILES);
    h->boxsize = get<double>(b, H_BOX);
    h->omega0 = get<double>(b, H_OM);
    h->omega_lambda = get<double>(b, H_OL);
    h->hubble = get<double>(b, H_H);
}

void encode(const photons_gadget_header *h, unsigned char *b)
{
    memset(b, 0, H_BYTES);
    for (int i = 0; i < 6; i++) {
        put<int>(b, H_NPART + 4 * i, h->npart[i]);
        put<double>(b, H_MASS + 8 * i, h->mass[i]);
        put<int>(b, H_NTOTAL + 4 * i, h->npart_total[i]);
    }
    put<double>(b, H_TIME, h->time);
    put<double>(b, H_REDSHIFT, h->redshift);
    put<int>(b, H_SFR, h->flag_sfr);
    put<int>(b, H_FEEDBACK, h->flag_feedback);
    put<int>(b, H_COOLING, h->flag_cooling);
    put<int>(b, H_NFILES, h->num_files);
    put<double>(b, H_BOX, h->boxsize);
    put<double>(b, H_OM, h->omega0);
    put<double>(b, H_OL, h->omega_lambda);
    put<double>(b, H_H, h->hubble);
}

struct File {
    FILE *f = nullptr;
    ~File()
    {
        if (f) fclose(f);
    }
};

int read_marker(FILE *f, int *v) { return fread(v, sizeof(int), 1, f) == 1 ? 0 : -1; }

long long file_particles(const photons_gadget_header &h)
{
    long long n = 0;
    for (int i = 0; i < 6; i++) n += h.npart[i];
    return n;
}

// one block of n float triples, records of 4 bytes around it
int read_block(FILE *f, long long n, long long first, long long count, double *out, double scale, const char *what)
{
    // the record markers are skipped unread: the reference's writer leaves
    // them uninitialised (src/snapshot.c:452-485)
    int m0 = 0, m1 = 0;
    if (read_marker(f, &m0)) return ph_set_error(PH_ERR_ARG, "snapshot: truncated before the %s block", what);
    std::vector<float> buf(3 * (size_t)(n > 0 ? n : 1));
    if (n > 0 && fread(buf.data(), sizeof(float), 3 * (size_t)n, f) != 3 * (size_t)n)
        return ph_set_error(PH_ERR_ARG, "snapshot: truncated %s block", what);
    if (read_marker(f, &m1)) return ph_set_error(PH_ERR_ARG, "snapshot: truncated after the %s block", what);
    for (long long i = 0; i < count; i++)
        for (int d = 0; d < 3; d++) {
            const double v = (double)buf[3 * (size_t)(first + i) + d];
            out[3 * i + d] = scale == 1.0 ? v : v * scale;
        }
    return 0;
}

}  // namespace

extern "C" int photons_gadget_read_header(const char *path, photons_gadget_header *h)
{
    photons_gpu_clear_error();
    if (!path || !h) return ph_set_error(PH_ERR_ARG, "null argument");
    File fh;
    if (!(fh.f = fopen(path, "rb"))) return ph_set_error(PH_ERR_ARG, "cannot open snapshot %s", path);
    int m0 = 0, m1 = 0;
    unsigned char b[H_BYTES];
    if (read_marker(fh.f, &m0) || fread(b, 1, H_BYTES, fh.f) != H_BYTES || read_marker(fh.f, &m1))
        return ph_set_error(PH_ERR_ARG, "snapshot %s: truncated header", path);
    decode(b, h);
    return 0;
}

extern "C" int photons_gadget_read(const char *path, long long first, long long count, double *pos, double *vel)
{
    photons_gpu_clear_error();
    photons_gadget_header h;
    PH_TRY(photons_gadget_read_header(path, &h));
    const long long n = file_particles(h);
    if (first < 0 || count < 0 || first + count > n)
        return ph_set_error(PH_ERR_ARG, "snapshot %s holds %lld particles; asked for [%lld, %lld)", path, n, first,
                            first + count);
    File fh;
    if (!(fh.f = fopen(path, "rb"))) return ph_set_error(PH_ERR_ARG, "cannot open snapshot %s", path);
    if (fseek(fh.f, 4 + H_BYTES + 4, SEEK_SET)) return ph_set_error(PH_ERR_ARG, "snapshot %s: seek failed", path);
    std::vector<double> scratch;
    double *p = pos;
    if (!p) {
        scratch.resize(3 * (size_t)(count > 0 ? count : 1));
        p = scratch.data();
    }
    PH_TRY(read_block(fh.f, n, first, count, p, 1.0, "position"));
    if (vel) {
        const double gdt2unit = pow(1.0 / (1.0 + h.redshift), 1.5);
        PH_TRY(read_block(fh.f, n, first, count, vel, gdt2unit, "velocity"));
    }
    return 0;
}

extern "C" int photons_gadget_write(const char *path, const photons_gadget_header *h, long long n, const double *pos,
                                    const double *vel)
{
    photons_gpu_clear_error();
    if (!path || !h || n < 0 || (n > 0 && (!pos || !vel))) return ph_set_error(PH_ERR_ARG, "bad snapshot arguments");
    if (n * 12 > 0x7fffffffLL) return ph_set_error(PH_ERR_ARG, "snapshot block of %lld particles exceeds 2 GB", n);
    File fh;
    if (!(fh.f = fopen(path, "wb"))) return ph_set_error(PH_ERR_ARG, "cannot create snapshot %s", path);
    unsigned char b[H_BYTES];
    encode(h, b);
    const int hm = H_BYTES, bm = (int)(n * 12);
    bool ok = fwrite(&hm, 4, 1, fh.f) == 1 && fwrite(b, 1, H_BYTES, fh.f) == H_BYTES && fwrite(&hm, 4, 1, fh.f) == 1;
    std::vector<float> buf(3 * (size_t)(n > 0 ? n : 1));
    for (long long i = 0; i < 3 * n; i++) buf[i] = (float)pos[i];
    ok = ok && fwrite(&bm, 4, 1, fh.f) == 1 && fwrite(buf.data(), sizeof(float), 3 * (size_t)n, fh.f) == 3 * (size_t)n &&
         fwrite(&bm, 4, 1, fh.f) == 1;
    const double gdt2unit = pow(1.0 / (1.0 + h->redshift), 1.5);
    for (long long i = 0; i < 3 * n; i++) buf[i] = (float)vel[i] / gdt2unit;
    ok = ok && fwrite(&bm, 4, 1, fh.f) == 1 && fwrite(buf.data(), sizeof(float), 3 * (size_t)n, fh.f) == 3 * (size_t)n &&
         fwrite(&bm, 4, 1, fh.f) == 1;
    if (!ok) return ph_set_error(PH_ERR_ARG, "snapshot %s: write failed", path);
    return 0;
}
