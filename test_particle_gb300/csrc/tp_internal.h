// tp_internal.h -- library-private state shared by the host translation units.
#pragma once
#include <vector>

#include "tp_common.cuh"

namespace tp {

// Device copy of one caller-owned host array.  device_only: the device copy is
// authoritative (filled on the GPU, e.g. synthesised fields) and never uploaded.
struct Mirror {
    const void* src = nullptr;
    size_t bytes = 0, cap = 0;
    void* dev = nullptr;
    bool dirty = true;
    bool device_only = false;
    bool sync(const void* host, size_t b, cudaStream_t s);
    void release();
};

// Grow-only device scratch buffer.
struct Scratch {
    void* ptr = nullptr;
    size_t cap = 0;
    void* get(size_t b);
    void release();
};

struct Ctx {
    bool inited = false;
    int device = 0;
    int num_sms = 0;
    cudaStream_t stream = nullptr;
    int* d_status = nullptr;
    int status = 0;
    char err[512] = {0};
    // ABC coefficients: compile-time macros in the reference (include/force_free.h:21-26)
    double ffA = 1.0, ffB = 0.81649658092772603, ffC = 0.57735026918962573;
    int interp_corrected = 0, ellint_corrected = 0;
    unsigned int wait_limit = 0;  // tensor-core pipeline hand-over polls (0: default)
    int compact_steps = -1;       // open-boundary segment length (0: off, -1: automatic)
    std::vector<tp_mode> modes;
    double mode_B0 = 1.0;
    long modes_gen = 0;
    // mirrors of the reference's host grids
    Mirror m_bc_f, m_ba_f, m_bb_f, m_ec_f, m_ea_f, m_eb_f, m_vc_f, m_va_f, m_vb_f;
    Mirror m_bc_d, m_ba_d, m_bb_d, m_ec_d, m_ea_d, m_eb_d, m_vc_d, m_va_d, m_vb_d;
    Mirror m_cfg, m_modes;
    std::vector<Mirror*> all_mirrors()
    {
        return {&m_bc_f, &m_ba_f, &m_bb_f, &m_ec_f, &m_ea_f, &m_eb_f, &m_vc_f, &m_va_f, &m_vb_f,
                &m_bc_d, &m_ba_d, &m_bb_d, &m_ec_d, &m_ea_d, &m_eb_d, &m_vc_d, &m_va_d, &m_vb_d,
                &m_cfg, &m_modes};
    }
    // exact energy-bin thresholds on the device
    int thr_nbins = 0;
    double thr_logemin = 0.0, thr_logde = 0.0;
    double* d_thr = nullptr;
    // scratch for batch utilities
    Scratch s_batch_a, s_batch_b;
    // mixed-precision field copies (FP32 node-interleaved grids, FP32 modes)
    Scratch s_mix_v, s_mix_eb, s_mix_modes;
    const float* eb_src_e = nullptr;
    const float* eb_src_b = nullptr;
    size_t eb_n = 0;
    long eb_gen = -1;
    long upload_gen = 0;     // bumped by every host-to-device field upload
};

extern Ctx g;

void set_error(int code, const char* fmt, ...);
bool cuda_ok(cudaError_t e, const char* what);
void die_if_error(const char* where);
bool ensure_init();
bool build_field(int stype, DevField& f);
bool build_field_points(DevField& f);
namespace mixed { struct MixField; }
bool build_mixfield(int stype, mixed::MixField& mf, int* nmodes_out);
const void* dd0(Mirror& m, const void* h, size_t b, cudaStream_t s);
bool ensure_thresholds(int nbins);
bool compute_thresholds(int nbins, double lmin, double lde, std::vector<double>& thr);
void aos_to_soa(const double* d_aos, int n, double* d_soa, long stride, cudaStream_t s);
void soa_to_aos(const double* d_soa, int n, long stride, double* d_aos, cudaStream_t s);

}  // namespace tp
