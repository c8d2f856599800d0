// mcd_host.cpp - host-only entry points of libmcd: material constants,
// error strings, layout queries and device information.
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>
#include <string.h>

#include "../../include/mcd.h"

namespace {

// CODATA 2022 values (scipy.constants as the reference uses them)
constexpr double kAvogadro = 6.02214076e23;
constexpr double kHbar = 1.0545718176461565e-34;
constexpr double kMe = 9.1093837139e-31;
constexpr double kE = 1.602176634e-19;
constexpr double kEps0 = 8.8541878188e-12;
constexpr double kPi = 3.141592653589793;

struct ShellSpec {
    const char* name;
    double E;
    double n;
};

struct SpeciesSpec {
    const char* species;
    const char* name_val;
    int Z;
    double n_val, E_val, density, atwt, bethe_k;
    double xip_g;  // extinction distance (0,0,4) at 20 keV, material.py:225-226; 0 = none
    int n_shells;
    ShellSpec shells[MCD_MAX_SHELLS];
};

// MC/tools/material.py:151-302 (shell order = the reference's name_s order)
const SpeciesSpec kSpecies[] = {
    {"Al", "3s2-3p1", 13, 3, 72.55, 2.70, 26.98154, 0.815, 0.0, 3,
     {{"1s", 1559.0, 2}, {"2s", 118.0, 2}, {"2p", 73.5, 6}}},
    {"Si", "3s2-3p2", 14, 4, 99.42, 2.33, 28.085, 0.822, 1360.0, 3,
     {{"1s", 1189.0, 2}, {"2s", 149.0, 2}, {"2p", 100.0, 6}}},
    {"Cu", "3d10-4s2", 29, 11, 75.1, 8.96, 63.546, 0.83, 0.0, 4,
     {{"1s", 8980.0, 2}, {"2s2p", 977.0, 8}, {"3s", 120.0, 2}, {"3p", 74.0, 6}}},
    {"Au", "5d10-6s1", 79, 11, 75.1, 19.30, 196.967, 0.851, 0.0, 8,
     {{"2s2p", 12980.0, 8}, {"3s3p3d", 2584.0, 18}, {"4s4p", 624.0, 8}, {"4d", 341.0, 10},
      {"5s", 178.0, 2}, {"4f", 85.0, 14}, {"5p2", 72.0, 2}, {"5p4", 54.0, 4}}},
};

void copy_name(char* dst, size_t cap, const char* src) {
    snprintf(dst, cap, "%s", src);
}

}  // namespace

extern "C" int mcd_abi_version(void) { return MCD_ABI_VERSION; }

extern "C" size_t mcd_event_bytes(uint32_t fields) {
    uint32_t f = fields & MCD_EV_ALL;
    if (f == 0) f = MCD_EV_ALL;
    const size_t head = (fields & MCD_EV_PACKED_HEAD) ? 1 : 2;
    size_t words = head + (size_t)__builtin_popcount(f & 0x1fu) + ((f & MCD_EV_POS) ? 3 : 0);
    return 4 * words;
}

extern "C" const char* mcd_strerror(int code) {
    switch (code) {
        case MCD_OK: return "ok";
        case MCD_EINVAL: return "invalid argument";
        case MCD_ECUDA: return "CUDA runtime error";
        case MCD_ETOOBIG: return "size beyond a documented limit";
        case MCD_ENOSPECIES: return "unknown material (Al, Si, Cu, Au are defined)";
        case MCD_ENODEV: return "no CUDA device";
        default: return "unknown error code";
    }
}

extern "C" size_t mcd_struct_size(const char* name) {
    if (!name) return 0;
    if (!strcmp(name, "mcd_material")) return sizeof(mcd_material);
    if (!strcmp(name, "mcd_table")) return sizeof(mcd_table);
    if (!strcmp(name, "mcd_sim")) return sizeof(mcd_sim);
    if (!strcmp(name, "mcd_tally")) return sizeof(mcd_tally);
    if (!strcmp(name, "mcd_electron_out")) return sizeof(mcd_electron_out);
    if (!strcmp(name, "mcd_event")) return sizeof(mcd_event);
    if (!strcmp(name, "mcd_event_ring")) return sizeof(mcd_event_ring);
    if (!strcmp(name, "mcd_tune")) return sizeof(mcd_tune);
    if (!strcmp(name, "mcd_softhist")) return sizeof(mcd_softhist);
    if (!strcmp(name, "mcd_adjoint_buf")) return sizeof(mcd_adjoint_buf);
    return 0;
}

// material.py:15-90 (atomic number density, plasmon and Fermi energies) and
// stoppingPowers.py:134-137 (mean ionisation energy J from Z)
extern "C" int mcd_material_init(const char* species, mcd_material* out) {
    if (!species || !out) return MCD_EINVAL;
    const SpeciesSpec* s = nullptr;
    for (const auto& sp : kSpecies)
        if (!strcmp(sp.species, species)) s = &sp;
    if (!s) return MCD_ENOSPECIES;
    memset(out, 0, sizeof(*out));
    copy_name(out->species, sizeof(out->species), s->species);
    copy_name(out->name_val, sizeof(out->name_val), s->name_val);
    out->Z = s->Z;
    out->n_shells = s->n_shells;
    out->n_val = s->n_val;
    out->E_val = s->E_val;
    out->density = s->density;
    out->atwt = s->atwt;
    out->bethe_k = s->bethe_k;
    out->xip_g = s->xip_g;
    for (int k = 0; k < s->n_shells; ++k) {
        copy_name(out->shell_name[k], sizeof(out->shell_name[k]), s->shells[k].name);
        out->shell_E[k] = s->shells[k].E;
        out->shell_n[k] = s->shells[k].n;
    }
    out->atnd = s->density * kAvogadro / s->atwt * 1e6;
    const double nv = s->n_val * out->atnd;
    out->plasmon_e = kHbar * kE * sqrt(nv / (kEps0 * kMe)) / kE;
    out->fermi_e = kHbar * kHbar * pow(3.0 * kPi * kPi * nv, 2.0 / 3.0) / (2.0 * kMe) / kE;
    const double Z = (double)s->Z;
    out->J = (s->Z >= 13) ? (9.76 * Z + 58.5 / pow(Z, 0.19)) : 11.5 * Z;
    return MCD_OK;
}

extern "C" int mcd_device_info(int* sm_count, int* cc_major, int* cc_minor) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n < 1) return MCD_ENODEV;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return MCD_ECUDA;
    if (sm_count && cudaDeviceGetAttribute(sm_count, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        return MCD_ECUDA;
    if (cc_major && cudaDeviceGetAttribute(cc_major, cudaDevAttrComputeCapabilityMajor, dev) != cudaSuccess)
        return MCD_ECUDA;
    if (cc_minor && cudaDeviceGetAttribute(cc_minor, cudaDevAttrComputeCapabilityMinor, dev) != cudaSuccess)
        return MCD_ECUDA;
    return MCD_OK;
}
