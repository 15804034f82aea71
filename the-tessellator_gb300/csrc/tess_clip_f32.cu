// tess_clip_f32.cu -- FP32 instantiations of the clipping kernel (the
// FP32 + FP64-guard form); kernel source in tess_clip_impl.cuh.
#include "tess_clip_impl.cuh"

namespace tess {

cudaError_t launch_clip_f32(const ClipParams& p, int slots, int form, int wpb, int blocks, cudaStream_t s) {
    using namespace clipk;
    const bool geo = p.geo != nullptr;
    if (slots <= 2) {
        if (geo) return launch_t<float, 2, true, kFormStd>(p, wpb, blocks, s);
        if (form == kFormHybrid) return launch_t<float, 2, false, kFormHybrid>(p, wpb, blocks, s);
        return form == kFormLean ? launch_t<float, 2, false, kFormLean>(p, wpb, blocks, s)
                                 : launch_t<float, 2, false, kFormStd>(p, wpb, blocks, s);
    }
    if (slots <= 4)
        return geo ? launch_t<float, 4, true, kFormStd>(p, wpb, blocks, s) : launch_t<float, 4, false, kFormStd>(p, wpb, blocks, s);
    return geo ? launch_t<float, 8, true, kFormStd>(p, wpb, blocks, s) : launch_t<float, 8, false, kFormStd>(p, wpb, blocks, s);
}

int clip_blocks_f32(int slots, int form, int wpb, int device) {
    using namespace clipk;
    if (slots <= 2) {
        if (form == kFormHybrid) return blocks_t<float, 2, false, kFormHybrid>(wpb, device);
        return form == kFormLean ? blocks_t<float, 2, false, kFormLean>(wpb, device)
                                 : blocks_t<float, 2, false, kFormStd>(wpb, device);
    }
    if (slots <= 4) return blocks_t<float, 4, false, kFormStd>(wpb, device);
    return blocks_t<float, 8, false, kFormStd>(wpb, device);
}

}  // namespace tess
