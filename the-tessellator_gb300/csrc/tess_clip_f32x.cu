// tess_clip_f32x.cu -- FP32 instantiations with the FP64-accurate finish
// (kFormExact, TESS_PRECISION_MIXED); a translation unit of its own so the
// build compiles it beside tess_clip_f32.cu.  Kernel source in
// tess_clip_impl.cuh.
#include "tess_clip_impl.cuh"

namespace tess {

cudaError_t launch_clip_f32x(const ClipParams& p, int slots, int form, int wpb, int blocks, cudaStream_t s) {
    using namespace clipk;
    const int base = form & 3;
    if (slots <= 2) {
        if (base == kFormHybrid) return launch_t<float, 2, false, kFormHybrid | kFormExact>(p, wpb, blocks, s);
        return base == kFormLean ? launch_t<float, 2, false, kFormLean | kFormExact>(p, wpb, blocks, s)
                                 : launch_t<float, 2, false, kFormStd | kFormExact>(p, wpb, blocks, s);
    }
    if (slots <= 4) return launch_t<float, 4, false, kFormStd | kFormExact>(p, wpb, blocks, s);
    return launch_t<float, 8, false, kFormStd | kFormExact>(p, wpb, blocks, s);
}

int clip_blocks_f32x(int slots, int form, int wpb, int device) {
    using namespace clipk;
    const int base = form & 3;
    if (slots <= 2) {
        if (base == kFormHybrid) return blocks_t<float, 2, false, kFormHybrid | kFormExact>(wpb, device);
        return base == kFormLean ? blocks_t<float, 2, false, kFormLean | kFormExact>(wpb, device)
                                 : blocks_t<float, 2, false, kFormStd | kFormExact>(wpb, device);
    }
    if (slots <= 4) return blocks_t<float, 4, false, kFormStd | kFormExact>(wpb, device);
    return blocks_t<float, 8, false, kFormStd | kFormExact>(wpb, device);
}

}  // namespace tess
