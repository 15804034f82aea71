// tess_clip_f32.cu -- FP32 instantiations of the clipping kernel (the
// FP32 + FP64-guard form, and with kFormExact its FP64-accurate finalize);
// kernel source in tess_clip_impl.cuh.
#include "tess_clip_impl.cuh"

namespace tess {

cudaError_t launch_clip_f32(const ClipParams& p, int slots, int form, int wpb, int blocks, cudaStream_t s) {
    using namespace clipk;
    const bool geo = p.geo != nullptr;
    const bool ex = (form & kFormExact) != 0;
    const int base = form & 3;
    if (slots <= 2) {
        if (geo) return launch_t<float, 2, true, kFormStd>(p, wpb, blocks, s);
        if (base == kFormHybrid)
            return ex ? launch_t<float, 2, false, kFormHybrid | kFormExact>(p, wpb, blocks, s)
                      : launch_t<float, 2, false, kFormHybrid>(p, wpb, blocks, s);
        if (base == kFormLean)
            return ex ? launch_t<float, 2, false, kFormLean | kFormExact>(p, wpb, blocks, s)
                      : launch_t<float, 2, false, kFormLean>(p, wpb, blocks, s);
        return ex ? launch_t<float, 2, false, kFormStd | kFormExact>(p, wpb, blocks, s)
                  : launch_t<float, 2, false, kFormStd>(p, wpb, blocks, s);
    }
    if (slots <= 4) {
        if (geo) return launch_t<float, 4, true, kFormStd>(p, wpb, blocks, s);
        return ex ? launch_t<float, 4, false, kFormStd | kFormExact>(p, wpb, blocks, s)
                  : launch_t<float, 4, false, kFormStd>(p, wpb, blocks, s);
    }
    if (geo) return launch_t<float, 8, true, kFormStd>(p, wpb, blocks, s);
    return ex ? launch_t<float, 8, false, kFormStd | kFormExact>(p, wpb, blocks, s)
              : launch_t<float, 8, false, kFormStd>(p, wpb, blocks, s);
}

int clip_blocks_f32(int slots, int form, int wpb, int device) {
    using namespace clipk;
    const bool ex = (form & kFormExact) != 0;
    const int base = form & 3;
    if (slots <= 2) {
        if (base == kFormHybrid)
            return ex ? blocks_t<float, 2, false, kFormHybrid | kFormExact>(wpb, device)
                      : blocks_t<float, 2, false, kFormHybrid>(wpb, device);
        if (base == kFormLean)
            return ex ? blocks_t<float, 2, false, kFormLean | kFormExact>(wpb, device)
                      : blocks_t<float, 2, false, kFormLean>(wpb, device);
        return ex ? blocks_t<float, 2, false, kFormStd | kFormExact>(wpb, device)
                  : blocks_t<float, 2, false, kFormStd>(wpb, device);
    }
    if (slots <= 4)
        return ex ? blocks_t<float, 4, false, kFormStd | kFormExact>(wpb, device)
                  : blocks_t<float, 4, false, kFormStd>(wpb, device);
    return ex ? blocks_t<float, 8, false, kFormStd | kFormExact>(wpb, device)
              : blocks_t<float, 8, false, kFormStd>(wpb, device);
}

}  // namespace tess
