// tess_clip_f32.cu -- FP32 instantiations of the clipping kernel (the
// FP32 + FP64-guard form); the forms with the FP64-accurate finish
// (kFormExact) are in tess_clip_f32x.cu.  Kernel source in tess_clip_impl.cuh.
#include "tess_clip_impl.cuh"

namespace tess {

cudaError_t launch_clip_f32x(const ClipParams& p, int slots, int form, int wpb, int blocks, cudaStream_t s);
int clip_blocks_f32x(int slots, int form, int wpb, int device);

cudaError_t launch_clip_f32(const ClipParams& p, int slots, int form, int wpb, int blocks, cudaStream_t s) {
    using namespace clipk;
    const bool geo = p.geo != nullptr;
    if ((form & kFormExact) && !geo) return launch_clip_f32x(p, slots, form, wpb, blocks, s);
    const int base = form & 3;
    if (slots <= 2) {
        if (geo) return launch_t<float, 2, true, kFormStd>(p, wpb, blocks, s);
        if (base == kFormHybrid) return launch_t<float, 2, false, kFormHybrid>(p, wpb, blocks, s);
        return base == kFormLean ? launch_t<float, 2, false, kFormLean>(p, wpb, blocks, s)
                                 : launch_t<float, 2, false, kFormStd>(p, wpb, blocks, s);
    }
    if (slots <= 4)
        return geo ? launch_t<float, 4, true, kFormStd>(p, wpb, blocks, s) : launch_t<float, 4, false, kFormStd>(p, wpb, blocks, s);
    return geo ? launch_t<float, 8, true, kFormStd>(p, wpb, blocks, s) : launch_t<float, 8, false, kFormStd>(p, wpb, blocks, s);
}

int clip_blocks_f32(int slots, int form, int wpb, int device) {
    using namespace clipk;
    if (form & kFormExact) return clip_blocks_f32x(slots, form, wpb, device);
    const int base = form & 3;
    if (slots <= 2) {
        if (base == kFormHybrid) return blocks_t<float, 2, false, kFormHybrid>(wpb, device);
        return base == kFormLean ? blocks_t<float, 2, false, kFormLean>(wpb, device)
                                 : blocks_t<float, 2, false, kFormStd>(wpb, device);
    }
    if (slots <= 4) return blocks_t<float, 4, false, kFormStd>(wpb, device);
    return blocks_t<float, 8, false, kFormStd>(wpb, device);
}

}  // namespace tess
