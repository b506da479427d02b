// context.h -- the library's context object, shared by the translation
// units of the C ABI (api.cu: buffers, NLCG, reparametrization; refine.cu:
// stationary-point refinement).  Internal; not part of include/mepgl.h.
#pragma once

#include <map>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/mepgl.h"
#include "kernels.cuh"

namespace mepgl {

// One string's host-side description and device buffers.
struct StringHost {
    int nx, ny, F;
    long M() const { return (long)nx * ny; }
    std::vector<double> params[9];     // a1 b1 mxx1 myy1 a2 b2 mxx2 myy2 h (host copy)
    std::vector<int32_t> comp, sc;
    bool uniform;
    void *dparams[9] = {};             // per-site arrays (type T) when not uniform
    uint16_t *dmask = nullptr;
    void *x[2][3] = {}, *g[2][3] = {}, *d[2][3] = {};
    double q[2], eta, gamma, delta, dx;
};

struct RefineWork;   // refine.cu
void refine_free(RefineWork *w);

}  // namespace mepgl

struct mepgl_ctx {
    int ncomp = 1, thin_film = 0, precision = 1;
    mepgl_options opt{};
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::vector<mepgl::StringHost> strings;
    std::vector<mepgl::StringDesc> hdesc;
    // strings are grouped MAX_STRINGS at a time; each group is one launch per
    // pass, its descriptors passed by value to the kernels
    std::vector<mepgl::Batch> batches;
    std::vector<int> batch_tile0, batch_ntiles, string_batch;
    mepgl::TileRef *dtiles = nullptr;
    int n_tiles = 0, total_images = 0;
    unsigned long long *fqueue = nullptr;   // work counter of the fused NLCG launch
    unsigned *fstage = nullptr;             // per-image stage counters of the fused NLCG launch
    std::vector<int> string_tile0, string_ntiles;
    mepgl::Scalars sc{};
    double *dscratch = nullptr;   // per-image temporaries (energies, 3 adjoints)
    double *ds = nullptr, *ds_jb = nullptr;   // arc lengths of string 0
    mepgl::RedistPlan plan{};
    int plan_cap = 0;
    void *cubic_scratch = nullptr;   // cubic resample columns of strings too long for shared memory
    size_t cubic_cap = 0;
    int xi = 0, di = 0;           // current x / d buffers
    bool pending = false;         // an NLCG update not yet applied to x
    int64_t launches = 0;
    std::string err;
    std::map<std::tuple<int, int, int, int>, cudaGraphExec_t> graphs;
    std::vector<double> host_s, host_sjb;
    int sm_count = 152;
    // staged state (mepgl_stage_state): a copy of the next state in flight on
    // a second stream while the context computes
    void *stage[3] = {nullptr, nullptr, nullptr};
    size_t stage_bytes = 0;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t stage_done = nullptr;
    bool staged = false;
    // workspace of mepgl_refine_stationary (refine.cu), allocated on first use
    mepgl::RefineWork *refine = nullptr;
    // bumped by every call that changes the fields other than the refinement
    // (which keeps per-state caches in its workspace)
    uint64_t state_version = 0;
};

namespace mepgl {

// Helpers of api.cu used by the other translation units.
// Record `msg` as the context's (or, for ctx == NULL, the thread's create) error.
mepgl_status ctx_fail(mepgl_ctx *c, mepgl_status st, const std::string &msg);
// Launch over the tiles of string si (its batch's descriptors).
Launch ctx_string_launch(mepgl_ctx *c, int si);
// Apply a pending NLCG update to x.
mepgl_status ctx_flush(mepgl_ctx *c);
// Read and clear the device status flags (see STATUS_* in kernels.cuh).
mepgl_status ctx_check_device_status(mepgl_ctx *c);

}  // namespace mepgl
