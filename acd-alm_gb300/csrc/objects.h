// The host objects behind approx_t and alm_t (shared by api.cu and
// static_solve.cu).
#pragma once
#include <mutex>
#include <vector>

#include "../../include/alm.h"
#include "../../include/approx.h"
#include "instance.h"
#include "layout.h"

struct approx {
        size_t nrhs = 0, nvars = 0;
        sparse_matrix_t * matrix = nullptr;  // borrowed
        sparse_matrix_t * permuted = nullptr;  // owned shadow copy
        // live vectors (the accessors' arrays)
        std::vector<double> rhs, weight, linear, lower, upper;
        // the shadow: what the last approx_update published
        std::vector<double> s_rhs, s_weight, s_linear, s_lower, s_upper;
        acd::DeviceLayout lay;
        bool lay_ready = false;
        // the step cap of the device layout built on first use: whole-GPU
        // solves by default; batches build theirs for one-CTA teams (0)
        int lay_max_steps = acd::grid_max_steps();
        acd::DevInstance dev;
        bool dev_ready = false;
        acd::SolveStats stats;
        std::mutex lock;
};

struct alm {
        size_t nrhs = 0, nvars = 0;
        sparse_matrix_t * matrix = nullptr;
        std::vector<double> linear, lambda_lower, lambda_upper;
        approx_t * approx = nullptr;
        acd::AlmSettings settings;
        acd::SolveStats stats;
};

struct acdalm_batch {
        std::vector<alm_t *> alms;
        double seconds = 0;
};
