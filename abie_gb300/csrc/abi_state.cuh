// The library's single simulation state (the reference keeps the same
// singleton on the host: struct Simulation, src/common.h:26-70).
#pragma once
#include <vector>

#include "force.cuh"

namespace abie {

struct Sim {
    bool inited = false;
    int dev = -1;
    int num_sms = 0;
    cudaStream_t st = nullptr;
    double G = 0.0, C = 0.0;
    size_t n_max = 0, n = 0;
    double t = 0.0;
    double ce_dist = 0.0;
    size_t max_ce = 0, max_coll = 0, n_ce = 0, n_coll = 0;
    std::vector<double> buf_ce, buf_coll;   // 4*max each: t, i, j, distance
    std::vector<double> h_m, h_r;           // host copies of masses and radii
    // device state (capacity n_max)
    double *pos = nullptr, *vel = nullptr, *m = nullptr, *r = nullptr, *ext_acc = nullptr;
    size_t pos_cap = 0, vel_cap = 0, m_cap = 0, r_cap = 0, ext_cap = 0;
    bool ext_enabled = false;
    // staging for the stateless host-array entry points
    double *tmp_pos = nullptr, *tmp_m = nullptr, *tmp_acc = nullptr, *tmp_vel = nullptr;
    size_t tmp_pos_cap = 0, tmp_m_cap = 0, tmp_acc_cap = 0, tmp_vel_cap = 0;
    double *energy_partials = nullptr;
    size_t energy_cap = 0;
    ForceScratch fs;
    int force_mode = ABIE_FORCE_FP64;
    abie_counters ctr = {};
};

extern Sim g_sim;

int ensure_device(int want);
int reserve(double **p, size_t *cap, size_t n);
void free_engine_buffers();

}  // namespace abie
