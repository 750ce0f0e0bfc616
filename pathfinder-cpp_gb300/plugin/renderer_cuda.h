// renderer_cuda.h - the reference-side drop-in: a SceneBuilder and a Renderer for
// pathfinder-cpp that hand the frame to libpfcuda.so (include/pfcuda.h).
//
// Compiled inside a pathfinder-cpp tree (it includes the reference's headers); it is the
// code a maintainer adds next to core/d3d9 and core/d3d11, with a new RenderMode case in
// Canvas::Canvas (pathfinder/core/canvas.cpp:157-171):
//
//     renderer = std::make_shared<RendererCuda>(device, queue);
//     scene_builder = std::make_shared<SceneBuilderCuda>();
//
// On a host with no graphics API the device and queue are the headless DeviceCuda::create()
// and QueueCuda of device_cuda.h.
//
// Canvas::draw (pathfinder/core/canvas.cpp:557-567) then calls
// scene_builder->build(scene, renderer) and renderer->draw(scene_builder, clear) as it does
// for the other modes.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "core/renderer.h"
#include "core/scene_builder.h"
#include "pfcuda.h"

namespace Pathfinder {

/// Packs the scene's draw paths and clip paths into the C-ABI's outline arrays
/// (SceneBuilder::build, pathfinder/core/scene_builder.h:16-27).  Replaces
/// SceneBuilderD3D11::build's segment packing (pathfinder/core/d3d11/scene_builder.cpp:209-223):
/// segments, bounds and tile rects are derived on the GPU.
class SceneBuilderCuda : public SceneBuilder {
public:
    void build(Scene *scene, Renderer *renderer) override;

    /// The packed scene; valid until the next build().
    const pf_scene_view &view() const {
        return view_;
    }

private:
    std::vector<float> points_;
    std::vector<uint8_t> flags_;
    std::vector<uint32_t> contour_start_, path_start_, color_, path_clip_;
    std::vector<uint8_t> fill_rule_, path_is_clip_;
    float view_box_[4] = {};
    pf_scene_view view_{};
};

/// Runs the GPU-driven frame on CUDA (Renderer, pathfinder/core/renderer.h:58-139).  The
/// RGBA8 result is written into the destination texture through the device's own command
/// encoder, so the rest of the application sees a normal Pathfinder texture.  draw() with
/// clear_dst_texture = false composites over the destination (LOAD_ACTION_LOAD,
/// core/d3d11/renderer.cpp:376-380): the pixels this renderer last wrote into it, handed back to
/// the frame with pf_write_image (the Device interface has no texture read-back).
class RendererCuda : public Renderer {
public:
    RendererCuda(const std::shared_ptr<Device> &device, const std::shared_ptr<Queue> &queue, int cuda_device = 0);
    ~RendererCuda() override;

    void set_up_pipelines() override {}

    std::shared_ptr<Texture> get_dest_texture() override {
        return dest_texture_;
    }

    void set_dest_texture(const std::shared_ptr<Texture> &texture) override {
        dest_texture_ = texture;
    }

    void draw(const std::shared_ptr<SceneBuilder> &scene_builder, bool clear_dst_texture) override;

    /// Loads learned-sizer weights; draw() then runs the learned one-pass frame wherever it
    /// measures faster than the exact one (pf_render_auto).
    bool load_sizer(const std::string &path);

    /// Statistics of the last frame.
    const pf_frame_stats &stats() const {
        return stats_;
    }

    /// The last frame's RGBA8 pixels (host copy).
    const std::vector<uint8_t> &pixels() const {
        return pixels_;
    }

protected:
    TextureFormat mask_texture_format() const override {
        return TextureFormat::Rgba8Unorm;  // no mask texture: coverage never leaves the SM
    }

private:
    void *ctx_ = nullptr;
    bool learned_ = false;
    std::shared_ptr<Texture> dest_texture_;
    pf_frame_stats stats_{};
    std::vector<uint8_t> pixels_;
};

}  // namespace Pathfinder
