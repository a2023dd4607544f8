// Shared by the translation units of the reference-side drop-in (GPUSpikingModel.cpp,
// bg3_classes.cpp, GpuSInput.cpp).  These files are compiled by g++ together with the reference's
// own host sources built with -DUSE_GPU and the reference's headers unchanged; they replace the
// reference's CUDA translation units (Core/GPUSpikingModel.cu, Neurons/*_d.cu, Synapses/*_d.cu,
// Connections/ConnGrowth_d.cu, Inputs/Gpu*.cu) and reach the GPU only through libbg3's C-ABI
// (include/bg3.h).
//
// Device structs become one opaque handle.  Where the reference passes `void* allNeuronsDevice`
// and `void* allSynapsesDevice` (device copies of its SoA structs) between the model and the
// neuron / synapse classes, this drop-in passes the network's bg3_net handle in both places:
// neurons, synapses, maps and the growth state of one network live in one bg3_net.
#ifndef BG3_DROPIN_H
#define BG3_DROPIN_H

#include <cstdio>
#include <cstdlib>
#include <vector>

#include "bg3.h"

// The reference's error convention (HANDLE_ERROR: message, then exit(EXIT_FAILURE)), applied to
// a bg3 status code.
inline void bg3_dropin_check(int rc, const char *what)
{
    if (rc != BG3_OK) {
        fprintf(stderr, "%s: %s (%d)\n", what, bg3_status_string(rc), rc);
        exit(EXIT_FAILURE);
    }
}

// The handle a device-struct pointer stands for; a NULL handle is a setup-order error.
inline bg3_net *bg3_dropin_net(void *device_struct, const char *what)
{
    if (!device_struct) {
        fprintf(stderr, "%s: no device network (GPUSpikingModel::setupSim creates it)\n", what);
        exit(EXIT_FAILURE);
    }
    return static_cast<bg3_net *>(device_struct);
}

// The network a GPUSpikingModel holds between setupSim and cleanupSim (NULL for any other model
// or outside that window); defined in GPUSpikingModel.cpp.
class IModel;
bg3_net *bg3_dropin_model_network(IModel *model);

// The spike-history ring between the reference's per-neuron rows (uint64_t *spike_history[N],
// each maxSpikes long) and the C-ABI's one row-major N x maxSpikes array.
inline void bg3_dropin_pack_history(uint64_t *const *rows, int n, int max_spikes,
                                    std::vector<uint64_t> &flat)
{
    flat.resize((size_t)n * (size_t)max_spikes);
    for (int i = 0; i < n; i++)
        for (int k = 0; k < max_spikes; k++) flat[(size_t)i * max_spikes + k] = rows[i][k];
}
inline void bg3_dropin_unpack_history(const std::vector<uint64_t> &flat, int n, int max_spikes,
                                      uint64_t *const *rows)
{
    for (int i = 0; i < n; i++)
        for (int k = 0; k < max_spikes; k++) rows[i][k] = flat[(size_t)i * max_spikes + k];
}

#endif
