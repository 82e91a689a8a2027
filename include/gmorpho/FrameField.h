// FrameField.h — opaque stand-in for the reference frame field
// (GMorpho/FrameField.h).  Rotated-cube dilation is not part of this
// library: GMorpho::Update with use_frame_field throws "unsupported".
#pragma once

namespace MorphoGraphics {
class FrameField {
 public:
  FrameField() {}
};
}  // namespace MorphoGraphics
