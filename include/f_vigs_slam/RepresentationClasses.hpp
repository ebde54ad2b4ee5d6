/*
 * f_vigs_slam/RepresentationClasses.hpp -- the reference's host-side types for
 * the hot path (include/f_vigs_slam/RepresentationClasses.hpp:101-141 of
 * jcevasco2003/f_vigs_slam), for the C++ mirror of GSSlam and
 * RgbdPoseCostFunction that sits on the fvgs C-ABI.
 *
 * CameraPose keeps the reference's layout and default (position float3,
 * orientation float4 built by the host as (w, x, y, z); identity
 * (1, 0, 0, 0)).  KeyframeData holds its images in host memory (the reference
 * keeps OpenCV GpuMats): 8-bit colour, 3 bytes per pixel in the camera's
 * (b, g, r) order, and depth in metres.
 */
#ifndef F_VIGS_SLAM_REPRESENTATION_CLASSES_HPP
#define F_VIGS_SLAM_REPRESENTATION_CLASSES_HPP

#include <cstdint>
#include <vector>

#include <vector_types.h>

namespace f_vigs_slam {

struct IntrinsicParameters {
    float2 f, c;
};

struct CameraPose {
    float3 position;
    float4 orientation;  // (w, x, y, z) as the reference's host builds it
    CameraPose() : position{0.0f, 0.0f, 0.0f}, orientation{1.0f, 0.0f, 0.0f, 0.0f} {}
    CameraPose(float3 pos, float4 quat) : position(pos), orientation(quat) {}
};

struct KeyframeData {
    std::vector<uint8_t> color_img;  // width x height x 3 bytes, (b, g, r)
    std::vector<float> depth_img;    // width x height, metres
    int width = 0, height = 0;
    CameraPose pose;
    IntrinsicParameters intrinsics{};
    uint32_t keyframe_id = 0;
    double timestamp = 0.0;

    const CameraPose& getPose() const { return pose; }
    void setPose(const CameraPose& p) { pose = p; }
    const IntrinsicParameters& getIntrinsics() const { return intrinsics; }
    int getWidth() const { return width; }
    int getHeight() const { return height; }
};

}  // namespace f_vigs_slam

#endif
