// Factoring a .cw wave list into the separable coefficient set.
//
// The volume solver writes (sCWatter.cpp:890-956), for each harmonic p (outer loop) of the
// M0 x M1 grid:
//   Pi        : the incident wave of p                          (not wound)
//   L0.Pr     : the reflected wave of p                         (wound to z_0)
//   L(l).Pt   : 2MF downward modes of slice l, per p             (wound to z_l),   l < Z
//   L(l).Pr   : 2MF upward modes of slice l-1, per p             (wound to z_l),   l >= 1
//   L(Z).Pt   : the transmitted wave of p                       (wound to z_Z)
// with kx = Sx(p) k, ky = Sy(p) k (p = a*M1 + b on the column-major flattening of the
// M1 x M0 mesh, so kx depends on a = p / M1 and ky on b = p % M1) and kz = gamma_j k.
// This file checks that structure exactly (equal kx per a, ky per b, kz per j across p)
// and re-references every amplitude to its own plane in FP64 before rounding to complex64.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstring>
#include <new>

#include "scw_sep.h"

using scw::fail;
using cd = std::complex<double>;

namespace {

inline cd rec_c(const double* r, int i) { return cd(r[2 * i], r[2 * i + 1]); }

}  // namespace

extern "C" {

scw_status scw_sep_info(scw_sep s, int* M0, int* M1, int* n_slices, int* modes_per_half) {
    if (!s) return fail(SCW_ERR_ARG, "null separable set");
    if (M0) *M0 = s->M0;
    if (M1) *M1 = s->M1;
    if (n_slices) *n_slices = s->Z;
    if (modes_per_half) *modes_per_half = s->J;
    return SCW_OK;
}

scw_status scw_sep_get_grid(scw_sep s, double* kx, double* ky, double* z_boundaries) {
    if (!s) return fail(SCW_ERR_ARG, "null separable set");
    if (kx) std::copy(s->kx.begin(), s->kx.end(), kx);
    if (ky) std::copy(s->ky.begin(), s->ky.end(), ky);
    if (z_boundaries) std::copy(s->zb.begin(), s->zb.end(), z_boundaries);
    return SCW_OK;
}

scw_status scw_sep_from_cw(scw_ctx ctx, scw_cw cw, scw_sep* out) {
    if (!ctx || !cw || !out) return fail(SCW_ERR_ARG, "scw_sep_from_cw: null argument");
    *out = nullptr;
    const size_t MF = cw->Pi.size() / 12;
    const size_t ZL = cw->layers.size();
    if (MF == 0 || ZL < 2) return fail(SCW_ERR_UNSUPPORTED, "not a volume-solver .cw (needs incident waves and >= 2 boundaries)");
    const int Z = (int)ZL - 1;
    // harmonic grid from the incident block
    const double* pi = cw->Pi.data();
    size_t M1 = 1;
    while (M1 < MF && pi[12 * M1 + 6] == pi[6] && pi[12 * M1 + 7] == pi[7]) M1++;
    if (MF % M1) return fail(SCW_ERR_UNSUPPORTED, "incident block is not an M0 x M1 harmonic grid");
    const size_t M0 = MF / M1;
    std::vector<double> kx(M0), ky(M1);
    for (size_t a = 0; a < M0; a++) kx[a] = pi[12 * (a * M1) + 6];
    for (size_t b = 0; b < M1; b++) ky[b] = pi[12 * b + 8];
    auto grid_ok = [&](const double* r, size_t p) {
        return r[6] == kx[p / M1] && r[7] == 0.0 && r[8] == ky[p % M1] && r[9] == 0.0;
    };
    for (size_t p = 0; p < MF; p++)
        if (!grid_ok(pi + 12 * p, p)) return fail(SCW_ERR_UNSUPPORTED, "incident kx/ky are not separable");
    const auto& L0 = cw->layers[0];
    const auto& LZ = cw->layers[ZL - 1];
    if (L0.Pr.size() != 12 * MF || LZ.Pt.size() != 12 * MF)
        return fail(SCW_ERR_UNSUPPORTED, "reflected / transmitted blocks are not one wave per harmonic");
    const size_t J = L0.Pt.size() / 12 / MF;
    if (L0.Pt.size() != 12 * MF * J) return fail(SCW_ERR_UNSUPPORTED, "slice-0 mode block is not MF x J");
    for (int l = 0; l < Z; l++) {
        const size_t npt = cw->layers[l].Pt.size(), npr = cw->layers[l + 1].Pr.size();
        if (npt != 12 * MF * J || npr != 12 * MF * J)
            return fail(SCW_ERR_UNSUPPORTED, "slice " + std::to_string(l) + " mode blocks are not MF x J");
    }
    std::vector<double> zb(ZL);
    for (size_t l = 0; l < ZL; l++) zb[l] = cw->layers[l].z;

    scw_sep s = nullptr;
    scw_status st = scw_sep_create(ctx, (int)M0, (int)M1, Z, (int)J, kx.data(), ky.data(), zb.data(), &s);
    if (st != SCW_OK) return st;

    // exterior blocks, each amplitude re-referenced to its block's plane
    std::vector<double> inc(6 * MF), refl(6 * MF), trans(6 * MF), kzi(2 * MF), kzr(2 * MF), kzt(2 * MF);
    auto fill = [&](const std::vector<double>& src, double zref, std::vector<double>& amp, std::vector<double>& kz) -> bool {
        for (size_t p = 0; p < MF; p++) {
            const double* r = src.data() + 12 * p;
            if (!grid_ok(r, p)) return false;
            const cd k = rec_c(r, 5);
            const cd f = std::exp(cd(0, 1) * k * zref);
            kz[2 * p] = k.real();
            kz[2 * p + 1] = k.imag();
            for (int c = 0; c < 3; c++) {
                const cd e = rec_c(r, c) * f;
                amp[2 * (c * MF + p)] = e.real();
                amp[2 * (c * MF + p) + 1] = e.imag();
            }
        }
        return true;
    };
    if (!fill(cw->Pi, 0.0, inc, kzi) || !fill(L0.Pr, zb[0], refl, kzr) || !fill(LZ.Pt, zb[ZL - 1], trans, kzt)) {
        scw_sep_destroy(s);
        return fail(SCW_ERR_UNSUPPORTED, "exterior waves are not separable");
    }
    st = scw_sep_set_exterior(s, inc.data(), kzi.data(), refl.data(), kzr.data(), trans.data(), kzt.data());
    if (st != SCW_OK) {
        scw_sep_destroy(s);
        return st;
    }
    if (J == 0) {
        *out = s;
        return SCW_OK;
    }
    // slices: Q[c][p][j] (complex64 on the device), kz per j
    std::vector<float2> qdn(3 * MF * J), qup(3 * MF * J);
    std::vector<double> kzdn(2 * J), kzup(2 * J);
    auto modes = [&](const std::vector<double>& src, double zref, std::vector<float2>& q, std::vector<double>& kz) -> bool {
        for (size_t j = 0; j < J; j++) {
            const double* r0 = src.data() + 12 * j;
            kz[2 * j] = r0[10];
            kz[2 * j + 1] = r0[11];
        }
        for (size_t p = 0; p < MF; p++) {
            for (size_t j = 0; j < J; j++) {
                const double* r = src.data() + 12 * (p * J + j);
                if (!grid_ok(r, p) || r[10] != kz[2 * j] || r[11] != kz[2 * j + 1]) return false;
                const cd f = std::exp(cd(0, 1) * rec_c(r, 5) * zref);
                for (int c = 0; c < 3; c++) {
                    const cd e = rec_c(r, c) * f;
                    q[(c * MF + p) * J + j] = make_float2((float)e.real(), (float)e.imag());
                }
            }
        }
        return true;
    };
    for (int l = 0; l < Z; l++) {
        if (!modes(cw->layers[l].Pt, zb[l], qdn, kzdn) || !modes(cw->layers[l + 1].Pr, zb[l + 1], qup, kzup)) {
            scw_sep_destroy(s);
            return fail(SCW_ERR_UNSUPPORTED, "slice " + std::to_string(l) + " waves are not separable");
        }
        st = scw_sep_set_slice_device(s, l, kzdn.data(), qdn.data(), kzup.data(), qup.data());
        if (st == SCW_OK) st = scw_ctx_synchronize(ctx);   // host buffers are reused next slice
        if (st != SCW_OK) {
            scw_sep_destroy(s);
            return st;
        }
    }
    *out = s;
    return SCW_OK;
}

}  // extern "C"
