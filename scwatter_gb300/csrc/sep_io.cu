// Compact factored coefficient file (.cwf): the separable set itself -- per slice the mode
// amplitudes Q_check / Q_hat (complex64) and the kz of the modes, plus the exterior blocks and
// the k grids -- instead of the reference's flat list of plane waves (CoupledWaveStructure.h:72-134).
// At MF = 1600 and 64 slices that is 15.7 GB (7.9 GB as a paired set) against the .cw file's ~63 GB, and the
// evaluator reads it without re-factoring.  Written and read slice by slice through a pinned
// staging buffer, so host memory stays at one slice.
//
// Layout (little-endian):
//   char[8]  "SCWSEP01" (two-half set) or "SCWSEP02" (paired set)
//   int32    M0, M1, Z, J (modes per half), rule (region rule), reserved (0)
//   float64  kx[M0], ky[M1], z_boundaries[Z + 1]
//   complex128 exterior[12 MF]     inc[3][MF], refl[3][MF], trans[3][MF], kz_inc, kz_refl, kz_trans
//   complex128 kz[Z][2][Jp]        Jp = J rounded up to even; entries J..Jp-1 are zero
//   SCWSEP01: complex64  Q[Z][2][3][MF][Jp]  amplitudes at the modes' reference planes
//   SCWSEP02: complex128 beta[Z][2][Jp], then complex64 V[Z][3][MF][Jp]: Q_dn = V diag(beta_dn),
//             Q_up = diag(1, 1, -1) V diag(beta_up) -- half the bytes of SCWSEP01
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "scw_internal.h"
#include "scw_sep.h"

using scw::fail;

namespace {

constexpr char kMagic[8] = {'S', 'C', 'W', 'S', 'E', 'P', '0', '1'};
constexpr char kMagicPaired[8] = {'S', 'C', 'W', 'S', 'E', 'P', '0', '2'};

struct File {
    FILE* f = nullptr;
    ~File() {
        if (f) fclose(f);
    }
};

struct Pinned {
    void* p = nullptr;
    ~Pinned() {
        if (p) cudaFreeHost(p);
    }
};

size_t q_slice_elems(const scw_sep_s* s) { return (size_t)s->halves * 3 * s->MF * s->Jp; }

}  // namespace

extern "C" {

scw_status scw_sep_save(scw_sep s, const char* path) {
    if (!s || !path) return fail(SCW_ERR_ARG, "scw_sep_save: null argument");
    SCW_ON_DEVICE(s->ctx->device);
    SCW_CUDA_TRY(cudaStreamSynchronize(s->ctx->stream));
    File out;
    out.f = fopen(path, "wb");
    if (!out.f) return fail(SCW_ERR_IO, std::string("cannot create ") + path);
    const int32_t hdr[6] = {s->M0, s->M1, s->Z, s->J, s->rule, 0};
    const size_t MF = (size_t)s->MF, kzn = (size_t)s->Z * 2 * s->Jp;
    const bool paired = s->halves == 1;
    std::vector<double2> ext(12 * MF), kz(kzn), beta(paired ? kzn : 0);
    SCW_CUDA_TRY(cudaMemcpy(ext.data(), s->dExt, sizeof(double2) * ext.size(), cudaMemcpyDeviceToHost));
    if (kzn) SCW_CUDA_TRY(cudaMemcpy(kz.data(), s->dKz, sizeof(double2) * kzn, cudaMemcpyDeviceToHost));
    if (paired && kzn) SCW_CUDA_TRY(cudaMemcpy(beta.data(), s->dBeta, sizeof(double2) * kzn, cudaMemcpyDeviceToHost));
    bool ok = fwrite(paired ? kMagicPaired : kMagic, 1, 8, out.f) == 8 && fwrite(hdr, sizeof(int32_t), 6, out.f) == 6 &&
              fwrite(s->kx.data(), 8, s->M0, out.f) == (size_t)s->M0 &&
              fwrite(s->ky.data(), 8, s->M1, out.f) == (size_t)s->M1 &&
              fwrite(s->zb.data(), 8, s->Z + 1, out.f) == (size_t)s->Z + 1 &&
              fwrite(ext.data(), sizeof(double2), ext.size(), out.f) == ext.size() &&
              fwrite(kz.data(), sizeof(double2), kzn, out.f) == kzn &&
              fwrite(beta.data(), sizeof(double2), beta.size(), out.f) == beta.size();
    const size_t qs = q_slice_elems(s);
    if (ok && s->dQ && s->Z > 0 && qs > 0) {
        Pinned buf;
        SCW_CUDA_TRY(cudaMallocHost(&buf.p, sizeof(float2) * qs));
        for (int l = 0; l < s->Z && ok; l++) {
            SCW_CUDA_TRY(cudaMemcpy(buf.p, s->dQ + (size_t)l * qs, sizeof(float2) * qs, cudaMemcpyDeviceToHost));
            ok = fwrite(buf.p, sizeof(float2), qs, out.f) == qs;
        }
    }
    if (!ok || fflush(out.f) != 0) return fail(SCW_ERR_IO, std::string("write failed: ") + path);
    return SCW_OK;
}

scw_status scw_sep_load(scw_ctx ctx, const char* path, scw_sep* out) {
    if (!ctx || !path || !out) return fail(SCW_ERR_ARG, "scw_sep_load: null argument");
    *out = nullptr;
    File in;
    in.f = fopen(path, "rb");
    if (!in.f) return fail(SCW_ERR_IO, std::string("cannot open ") + path);
    if (fseek(in.f, 0, SEEK_END) != 0) return fail(SCW_ERR_IO, std::string("cannot seek ") + path);
    const long long fsize = ftell(in.f);
    rewind(in.f);
    char magic[8];
    int32_t hdr[6];
    if (fread(magic, 1, 8, in.f) != 8 ||
        (std::memcmp(magic, kMagic, 8) != 0 && std::memcmp(magic, kMagicPaired, 8) != 0) || fread(hdr, 4, 6, in.f) != 6)
        return fail(SCW_ERR_FORMAT, std::string("not a factored coefficient file: ") + path);
    const bool paired = std::memcmp(magic, kMagicPaired, 8) == 0;
    const long long H = paired ? 1 : 2;
    const int M0 = hdr[0], M1 = hdr[1], Z = hdr[2], J = hdr[3], rule = hdr[4];
    if (M0 <= 0 || M1 <= 0 || Z < 0 || J < 0 || M0 > 4096 || M1 > 4096 || Z > (1 << 20) || J > (1 << 24))
        return fail(SCW_ERR_FORMAT, "factored file header out of range");
    const long long MF = (long long)M0 * M1, Jp = J + (J & 1);
    const long long need = 8 + 24 + 8LL * (M0 + M1 + Z + 1) + 16LL * 12 * MF + 16LL * Z * 2 * Jp * (paired ? 2 : 1) +
                           (J ? 8LL * Z * H * 3 * MF * Jp : 0);
    if (fsize != need) return fail(SCW_ERR_FORMAT, "factored file size does not match its header");
    std::vector<double> kx(M0), ky(M1), zb(Z + 1);
    if (fread(kx.data(), 8, M0, in.f) != (size_t)M0 || fread(ky.data(), 8, M1, in.f) != (size_t)M1 ||
        fread(zb.data(), 8, Z + 1, in.f) != (size_t)Z + 1)
        return fail(SCW_ERR_FORMAT, "truncated factored file");
    SCW_ON_DEVICE(ctx->device);
    scw_sep s = nullptr;
    scw_status st = paired ? scw_sep_create_paired(ctx, M0, M1, Z, J, kx.data(), ky.data(), zb.data(), &s)
                           : scw_sep_create(ctx, M0, M1, Z, J, kx.data(), ky.data(), zb.data(), &s);
    if (st != SCW_OK) return st;
    std::unique_ptr<scw_sep_s, scw_status (*)(scw_sep)> guard(s, scw_sep_destroy);
    s->rule = rule;
    std::vector<double2> ext(12 * MF), kz((size_t)Z * 2 * Jp), beta(paired ? (size_t)Z * 2 * Jp : 0);
    if (fread(ext.data(), sizeof(double2), ext.size(), in.f) != ext.size() ||
        fread(kz.data(), sizeof(double2), kz.size(), in.f) != kz.size() ||
        fread(beta.data(), sizeof(double2), beta.size(), in.f) != beta.size())
        return fail(SCW_ERR_FORMAT, "truncated factored file");
    SCW_CUDA_TRY(cudaMemcpy(s->dExt, ext.data(), sizeof(double2) * ext.size(), cudaMemcpyHostToDevice));
    if (!kz.empty()) SCW_CUDA_TRY(cudaMemcpy(s->dKz, kz.data(), sizeof(double2) * kz.size(), cudaMemcpyHostToDevice));
    if (!beta.empty())
        SCW_CUDA_TRY(cudaMemcpy(s->dBeta, beta.data(), sizeof(double2) * beta.size(), cudaMemcpyHostToDevice));
    const size_t qs = q_slice_elems(s);
    if (s->dQ && Z > 0 && qs > 0) {
        Pinned buf;
        SCW_CUDA_TRY(cudaMallocHost(&buf.p, sizeof(float2) * qs));
        for (int l = 0; l < Z; l++) {
            if (fread(buf.p, sizeof(float2), qs, in.f) != qs) return fail(SCW_ERR_FORMAT, "truncated factored file");
            SCW_CUDA_TRY(cudaMemcpy(s->dQ + (size_t)l * qs, buf.p, sizeof(float2) * qs, cudaMemcpyHostToDevice));
        }
    }
    *out = guard.release();
    return SCW_OK;
}

}  // extern "C"
