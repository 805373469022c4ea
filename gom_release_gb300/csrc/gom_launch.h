// gom_launch.h -- host-side launch interface between the ABI layer (gom_core.cu) and the kernel
// files.  Every launcher enqueues work on the context stream and returns a cudaError_t.
#pragma once

#include "gom_device.cuh"

namespace gom {

// device work buffers owned by a context
struct Work {
    // free surface / PCG
    double *sparsem = nullptr;   // (0:4, NC)
    double *rhs = nullptr;       // (NC)
    double *minv = nullptr, *r = nullptr, *s = nullptr, *q = nullptr, *d0 = nullptr, *d1 = nullptr;
    double *partial_dq = nullptr, *partial_delta = nullptr;   // (max_blocks)
    unsigned *barrier = nullptr;                               // [count, generation]
    int *pcg_iters = nullptr;                                  // device: iterations of the last solve
    int pcg_blocks = 0, pcg_threads = 256;
    // transport
    double *con = nullptr, *con2 = nullptr;   // (0:L+1, NC, 2)
    double *qj = nullptr, *dj = nullptr, *phij = nullptr;       // (L, NF)
    double *qi = nullptr, *di = nullptr, *phii = nullptr;       // (0:L, NC)
    double *psij = nullptr;                                     // (L, NF, 2)
    double *psii = nullptr;                                     // (0:L, NC, 2)
    double *sa1 = nullptr, *sa2 = nullptr;                      // (L, NC, 2) limiter sums per layer
    double *obk = nullptr, *qbk = nullptr;                      // (L, NOB, 2), (L, NQB, 2)
    // ELM: INT(dev/0.1) per (layer, face) edge
    int *idev = nullptr;
    // node velocities: face-level velocity / face length (0:L, NF), static node weights (NN)
    double *uflf = nullptr, *vflf = nullptr, *node_weight = nullptr;
    // conservation
    double *cons = nullptr;                                     // [volume, salt]
};

struct Launch {
    Geom g;
    State s;
    Forcing f;
    Params p;
    Work w;
    gom_status *status = nullptr;   // device
    cudaStream_t stream = nullptr;
    int num_sms = 0;
};

cudaError_t launch_bottom_friction(const Launch &x);
cudaError_t launch_boundary_velocity(const Launch &x);
cudaError_t launch_advection(const Launch &x);
cudaError_t launch_momentum(const Launch &x);
cudaError_t launch_free_surface(const Launch &x);
cudaError_t launch_velocities(const Launch &x);
cudaError_t launch_layers(const Launch &x);
cudaError_t launch_node_velocity(const Launch &x);
cudaError_t launch_transport(const Launch &x);
cudaError_t launch_density(const Launch &x);
cudaError_t launch_conservation(const Launch &x);

// cooperative PCG set-up (grid size from occupancy); called once per context
cudaError_t pcg_configure(Launch &x, int device);
// static per-node weights of calculate_velocity_at_node.f90:103; called once per context
cudaError_t launch_node_weights(const Launch &x);

}  // namespace gom
