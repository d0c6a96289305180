// vt_batch.cu — the batched solver: many isolated cloth domains advanced by the same
// multi-domain launches, one CUDA graph per frame.
#include <cstring>
#include <new>
#include <vector>

#include "vt_host.h"

using vt::HostSolver;

struct vt_batch {
    std::vector<HostSolver> doms;
    std::vector<uint64_t> offsets;  // first particle of each domain
    vt::World world;
    bool dirty = true;
    bool use_graph = true;
    cudaStream_t stream = nullptr;
    uint64_t launches_before = 0;
    // pipelined read-back (vt_batch_all_get_async): two packed buffers used in turn, each
    // with an event after its pack (compute stream) and after its copy (copy stream)
    float* rb_buf[2] = {nullptr, nullptr};
    size_t rb_floats = 0;
    cudaEvent_t rb_packed[2] = {nullptr, nullptr}, rb_copied[2] = {nullptr, nullptr};
    int rb_next = 0;

    ~vt_batch()
    {
        for (int k = 0; k < 2; ++k) {
            if (rb_buf[k]) cudaFree(rb_buf[k]);
            if (rb_packed[k]) cudaEventDestroy(rb_packed[k]);
            if (rb_copied[k]) cudaEventDestroy(rb_copied[k]);
        }
    }
};

#define VT_CHECK(cond, code, msg) \
    do {                          \
        if (!(cond)) {            \
            vt::set_error(msg);   \
            return code;          \
        }                         \
    } while (0)

#define VT_TRY_CUDA(call, what)                                \
    do {                                                       \
        cudaError_t e_ = (call);                               \
        if (e_ != cudaSuccess) return vt::cuda_fail(e_, what); \
    } while (0)

#define VT_GUARD_BEGIN try {
#define VT_GUARD_END                              \
    }                                             \
    catch (const std::bad_alloc&) {               \
        vt::set_error("host allocation failed");  \
        return VT_ERR_OUT_OF_MEMORY;              \
    }                                             \
    catch (...) {                                 \
        vt::set_error("unexpected host exception"); \
        return VT_ERR_STATE;                      \
    }

// Copies x, v, inverse mass of every domain back into the staging (before a rebuild).
static vt_status batch_pull(vt_batch* b)
{
    if (!b->world.built() || b->dirty) return VT_OK;
    VT_TRY_CUDA(cudaStreamSynchronize(b->stream), "sync");
    for (size_t k = 0; k < b->doms.size(); ++k) {
        HostSolver& h = b->doms[k];
        const size_t n = h.n(), o = b->offsets[k];
        if (!n) continue;
        VT_TRY_CUDA(cudaMemcpy2D(h.x.data(), 12, b->world.d.x + o, 16, 12, n, cudaMemcpyDeviceToHost), "pull x");
        VT_TRY_CUDA(cudaMemcpy2D(h.v.data(), 12, b->world.d.v + o, 16, 12, n, cudaMemcpyDeviceToHost), "pull v");
        VT_TRY_CUDA(cudaMemcpy2D(h.w.data(), 4, &b->world.d.x[o].w, 16, 4, n, cudaMemcpyDeviceToHost), "pull w");
    }
    return VT_OK;
}

extern "C" {

vt_status vt_batch_create(vt_batch** out)
{
    VT_CHECK(out, VT_ERR_INVALID_ARGUMENT, "out is NULL");
    VT_GUARD_BEGIN
    *out = new vt_batch();
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_batch_destroy(vt_batch* b)
{
    if (!b) return VT_OK;
    if (b->stream) cudaStreamSynchronize(b->stream);
    delete b;
    return VT_OK;
}

vt_status vt_batch_add(vt_batch* b, vt_solver* cloth, int32_t* out_index)
{
    VT_CHECK(b && cloth, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_GUARD_BEGIN
    vt::SolverImpl* s = cloth;
    vt_status st = vt::pull_state(s);
    if (st != VT_OK) return st;
    st = batch_pull(b);
    if (st != VT_OK) return st;
    b->doms.push_back(s->h);
    b->offsets.clear();
    uint64_t o = 0;
    for (const HostSolver& h : b->doms) {
        b->offsets.push_back(o);
        o += h.n();
    }
    b->dirty = true;
    if (out_index) *out_index = (int32_t)b->doms.size() - 1;
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_batch_size(const vt_batch* b, int32_t* num_cloths, uint64_t* num_particles)
{
    VT_CHECK(b, VT_ERR_INVALID_ARGUMENT, "NULL batch");
    if (num_cloths) *num_cloths = (int32_t)b->doms.size();
    if (num_particles) {
        uint64_t n = 0;
        for (const HostSolver& h : b->doms) n += h.n();
        *num_particles = n;
    }
    return VT_OK;
}

vt_status vt_batch_colliders_set(vt_batch* b, int32_t index, const vt_sdf_collider* c, uint32_t count)
{
    VT_CHECK(b, VT_ERR_INVALID_ARGUMENT, "NULL batch");
    VT_CHECK(index >= 0 && index < (int32_t)b->doms.size(), VT_ERR_NOT_FOUND, "no such cloth");
    VT_CHECK(count == 0 || c, VT_ERR_INVALID_ARGUMENT, "colliders is NULL");
    HostSolver& h = b->doms[index];
    VT_CHECK(count == h.colliders.size(), VT_ERR_INVALID_ARGUMENT,
             "a batched cloth keeps the collider count it was added with");
    for (uint32_t k = 0; k < count; ++k)
        VT_CHECK(c[k].type >= 0 && c[k].type <= 2, VT_ERR_INVALID_ARGUMENT, "unknown collider type");
    VT_GUARD_BEGIN
    h.colliders.assign(c, c + count);
    if (b->world.built() && !b->dirty) return b->world.set_colliders(index, h.colliders);
    return VT_OK;
    VT_GUARD_END
}

vt_status vt_batch_attach_slot_set(vt_batch* b, int32_t index, int32_t slot, const float xyz[3])
{
    VT_CHECK(b && xyz, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(index >= 0 && index < (int32_t)b->doms.size(), VT_ERR_NOT_FOUND, "no such cloth");
    HostSolver& h = b->doms[index];
    VT_CHECK(slot >= 0 && slot < (int32_t)h.nslots(), VT_ERR_INVALID_ARGUMENT, "slot out of range");
    for (int k = 0; k < 3; ++k) h.slots[3 * (size_t)slot + k] = xyz[k];
    if (b->world.built() && !b->dirty) {
        int32_t base = 0;
        for (int32_t k = 0; k < index; ++k) base += (int32_t)b->doms[k].nslots();
        return b->world.set_slot(index, base + slot, xyz);
    }
    return VT_OK;
}

vt_status vt_batch_simulate(vt_batch* b, float frame_dt, int32_t substeps, int32_t iterations,
                            float relaxation, float friction, float collision_margin,
                            const float* diameters, void* stream)
{
    VT_CHECK(b, VT_ERR_INVALID_ARGUMENT, "NULL batch");
    VT_CHECK(substeps >= 1 && iterations >= 0 && frame_dt > 0, VT_ERR_INVALID_ARGUMENT,
             "substeps must be >= 1, iterations >= 0, frame_dt > 0");
    if (b->doms.empty()) return VT_OK;
    const int32_t ih = b->doms[0].P.interleaved_hash;
    for (const HostSolver& h : b->doms)
        VT_CHECK(h.P.interleaved_hash == ih, VT_ERR_INVALID_ARGUMENT,
                 "all cloths of a batch must share interleaved_hash");
    VT_GUARD_BEGIN
    cudaStream_t st = (cudaStream_t)stream;
    if (b->dirty) {
        if (b->stream) VT_TRY_CUDA(cudaStreamSynchronize(b->stream), "sync");
        std::vector<const HostSolver*> doms;
        for (const HostSolver& h : b->doms) doms.push_back(&h);
        b->launches_before += b->world.launches;
        vt_status r = b->world.build(doms);
        if (r != VT_OK) return r;
        b->dirty = false;
    }
    b->stream = st;
    bool any_self = false;
    for (size_t k = 0; k < b->doms.size(); ++k) {
        HostSolver& h = b->doms[k];
        h.P.num_substeps = substeps;
        h.P.num_iterations = iterations;
        h.P.relaxation_factor = relaxation;
        h.P.friction = friction;
        h.P.collision_margin = collision_margin;
        if (diameters) h.P.particle_diameter = diameters[k];
        any_self = any_self || h.P.enable_self_collision;
        vt::FrameArgs a{frame_dt, substeps, iterations, relaxation, friction, collision_margin,
                        h.P.particle_diameter};
        b->world.set_frame((int)k, h, a);
    }
    vt::FrameArgs a{frame_dt, substeps, iterations, relaxation, friction, collision_margin, 0.0f};
    return b->world.simulate(a, ih, any_self, st, b->use_graph);
    VT_GUARD_END
}

vt_status vt_batch_sync(vt_batch* b)
{
    VT_CHECK(b, VT_ERR_INVALID_ARGUMENT, "NULL batch");
    VT_TRY_CUDA(cudaStreamSynchronize(b->stream), "sync");
    if (!b->world.built()) return VT_OK;
    std::vector<int32_t> flags;
    vt_status r = b->world.read_status(flags, b->stream);
    if (r != VT_OK) return r;
    if (flags[0]) {
        b->world.clear_status(b->stream);
        VT_TRY_CUDA(cudaStreamSynchronize(b->stream), "sync");
        if (flags[0] & vt::VT_STATUS_BOUNDS) {
            vt::set_error("a device-side bounds check failed (bounds-checked build)");
            return VT_ERR_STATE;
        }
        if (flags[0] & vt::VT_STATUS_TIMEOUT) {
            vt::set_error("a device-side bounded wait gave up (tile loads did not arrive)");
            return VT_ERR_TIMEOUT;
        }
        vt::set_error("non-finite particle state detected on the device");
        return VT_ERR_NUMERIC;
    }
    return VT_OK;
}

static vt_status batch_get(vt_batch* b, int32_t index, int which, float* dst, int32_t on_dev, void* stream)
{
    VT_CHECK(b && dst, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(index >= 0 && index < (int32_t)b->doms.size(), VT_ERR_NOT_FOUND, "no such cloth");
    VT_CHECK(b->world.built() && !b->dirty, VT_ERR_STATE, "state exists on the device after the first simulate");
    const size_t n = b->doms[index].n(), o = b->offsets[index];
    if (!n) return VT_OK;
    const float4* src = which == 0 ? b->world.d.x : which == 1 ? b->world.d.nrm : b->world.d.v;
    cudaStream_t st = (cudaStream_t)stream;
    float* pk = b->world.d.packed + 3 * o;
    VT_TRY_CUDA(vt::launch_pack_xyz(src + o, pk, (int64_t)n, st), "pack");
    b->world.launches += 1;
    VT_TRY_CUDA(cudaMemcpyAsync(dst, pk, 12 * n, on_dev ? cudaMemcpyDefault : cudaMemcpyDeviceToHost, st),
                "copy out");
    if (!on_dev) VT_TRY_CUDA(cudaStreamSynchronize(st), "sync");
    return VT_OK;
}

vt_status vt_batch_positions_get(vt_batch* b, int32_t index, float* dst, int32_t on_dev, void* stream)
{
    return batch_get(b, index, 0, dst, on_dev, stream);
}

vt_status vt_batch_normals_get(vt_batch* b, int32_t index, float* dst, int32_t on_dev, void* stream)
{
    return batch_get(b, index, 1, dst, on_dev, stream);
}

vt_status vt_batch_velocities_get(vt_batch* b, int32_t index, float* dst, int32_t on_dev, void* stream)
{
    return batch_get(b, index, 2, dst, on_dev, stream);
}

vt_status vt_batch_all_get(vt_batch* b, int32_t what, float* dst, int32_t on_dev, void* stream)
{
    VT_CHECK(b && dst, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(what >= 0 && what <= 2, VT_ERR_INVALID_ARGUMENT, "what must be 0, 1 or 2");
    VT_CHECK(b->world.built() && !b->dirty, VT_ERR_STATE, "state exists on the device after the first simulate");
    const size_t n = (size_t)b->world.n_particles;
    if (!n) return VT_OK;
    const float4* src = what == 0 ? b->world.d.x : what == 1 ? b->world.d.nrm : b->world.d.v;
    cudaStream_t st = (cudaStream_t)stream;
    VT_TRY_CUDA(vt::launch_pack_xyz(src, b->world.d.packed, (int64_t)n, st), "pack");
    b->world.launches += 1;
    VT_TRY_CUDA(cudaMemcpyAsync(dst, b->world.d.packed, 12 * n, on_dev ? cudaMemcpyDefault : cudaMemcpyDeviceToHost,
                                st),
                "copy out");
    if (!on_dev) VT_TRY_CUDA(cudaStreamSynchronize(st), "sync");
    return VT_OK;
}

vt_status vt_batch_all_get_async(vt_batch* b, int32_t what, float* dst, void* copy_stream)
{
    VT_CHECK(b && dst, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(what >= 0 && what <= 2, VT_ERR_INVALID_ARGUMENT, "what must be 0, 1 or 2");
    VT_CHECK(b->world.built() && !b->dirty, VT_ERR_STATE, "state exists on the device after the first simulate");
    const size_t n = (size_t)b->world.n_particles;
    if (!n) return VT_OK;
    if (b->rb_floats < 3 * n) {
        for (int k = 0; k < 2; ++k) {
            if (b->rb_buf[k]) VT_TRY_CUDA(cudaFree(b->rb_buf[k]), "cudaFree(read-back)");
            b->rb_buf[k] = nullptr;
        }
        b->rb_floats = 0;
        for (int k = 0; k < 2; ++k) {
            VT_TRY_CUDA(cudaMalloc(&b->rb_buf[k], 12 * n), "cudaMalloc(read-back)");
            if (!b->rb_packed[k])
                VT_TRY_CUDA(cudaEventCreateWithFlags(&b->rb_packed[k], cudaEventDisableTiming), "event");
            if (!b->rb_copied[k])
                VT_TRY_CUDA(cudaEventCreateWithFlags(&b->rb_copied[k], cudaEventDisableTiming), "event");
        }
        b->rb_floats = 3 * n;
    }
    const int k = b->rb_next;
    b->rb_next ^= 1;
    const float4* src = what == 0 ? b->world.d.x : what == 1 ? b->world.d.nrm : b->world.d.v;
    cudaStream_t cs = b->stream, xs = (cudaStream_t)copy_stream;
    // the buffer's previous copy has left it; the pack sees every frame enqueued so far
    VT_TRY_CUDA(cudaStreamWaitEvent(cs, b->rb_copied[k], 0), "wait copy");
    VT_TRY_CUDA(vt::launch_pack_xyz(src, b->rb_buf[k], (int64_t)n, cs), "pack");
    b->world.launches += 1;
    VT_TRY_CUDA(cudaEventRecord(b->rb_packed[k], cs), "event");
    VT_TRY_CUDA(cudaStreamWaitEvent(xs, b->rb_packed[k], 0), "wait pack");
    VT_TRY_CUDA(cudaMemcpyAsync(dst, b->rb_buf[k], 12 * n, cudaMemcpyDefault, xs), "copy out");
    VT_TRY_CUDA(cudaEventRecord(b->rb_copied[k], xs), "event");
    return VT_OK;
}

vt_status vt_batch_render(vt_batch* b, const vt_render_params* rp, uint32_t* rgba, int32_t dst_on_device,
                          void* stream)
{
    VT_CHECK(b && rp && rgba, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    VT_CHECK(vt::render_params_valid(*rp), VT_ERR_INVALID_ARGUMENT, "invalid render parameters");
    VT_CHECK(b->world.built() && !b->dirty, VT_ERR_STATE, "render after the first simulate");
    return vt::render_to(b->world.d.x, (int64_t)b->world.n_particles, *rp, rgba, dst_on_device != 0,
                         (cudaStream_t)stream, &b->world.launches);
}

vt_status vt_batch_launch_count(const vt_batch* b, uint64_t* out)
{
    VT_CHECK(b && out, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    *out = b->launches_before + b->world.launches;
    return VT_OK;
}

vt_status vt_batch_grid_tile(const vt_batch* b, int32_t* variant)
{
    VT_CHECK(b && variant, VT_ERR_INVALID_ARGUMENT, "NULL argument");
    *variant = b->world.grid_variant;
    return VT_OK;
}

vt_status vt_batch_use_graphs(vt_batch* b, int32_t on)
{
    VT_CHECK(b, VT_ERR_INVALID_ARGUMENT, "NULL batch");
    b->use_graph = on != 0;
    return VT_OK;
}

}  // extern "C"
