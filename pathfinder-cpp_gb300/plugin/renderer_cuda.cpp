// renderer_cuda.cpp - see renderer_cuda.h.
#include "renderer_cuda.h"

#include <cmath>

#include "common/logger.h"
#include "core/scene.h"

namespace Pathfinder {

void SceneBuilderCuda::build(Scene *scene, Renderer *renderer) {
    this->scene = scene;
    points_.clear();
    flags_.clear();
    contour_start_.assign(1, 0);
    path_start_.assign(1, 0);
    color_.clear();
    fill_rule_.clear();
    path_clip_.clear();
    path_is_clip_.clear();
    auto push_outline = [&](const Outline &outline) {
        for (const Contour &contour : outline.contours) {
            for (size_t i = 0; i < contour.points.size(); i++) {
                points_.push_back(contour.points[i].x);
                points_.push_back(contour.points[i].y);
                flags_.push_back(static_cast<uint8_t>(contour.flags[i]));
            }
            contour_start_.push_back(static_cast<uint32_t>(flags_.size()));
        }
        path_start_.push_back(static_cast<uint32_t>(contour_start_.size() - 1));
    };
    // draw paths, then the clip paths (Scene::clip_paths) after them; a draw path's clip
    // (DrawPath::clip_path) names its clip path by its index among all paths
    const uint32_t n_draw = static_cast<uint32_t>(scene->draw_paths.size());
    for (const DrawPath &path : scene->draw_paths) {
        push_outline(path.outline);
        const ColorU c = scene->get_paint(path.paint).get_base_color();
        color_.push_back(uint32_t(c.r_) | uint32_t(c.g_) << 8 | uint32_t(c.b_) << 16 | uint32_t(c.a_) << 24);
        fill_rule_.push_back(path.fill_rule == FillRule::EvenOdd ? PF_FILL_EVEN_ODD : PF_FILL_NONZERO);
        path_clip_.push_back(path.clip_path ? n_draw + *path.clip_path : PF_NO_CLIP);
        path_is_clip_.push_back(0);
    }
    for (const ClipPath &clip : scene->clip_paths) {
        push_outline(clip.outline);
        color_.push_back(0xffffffffu);  // never drawn
        fill_rule_.push_back(clip.fill_rule == FillRule::EvenOdd ? PF_FILL_EVEN_ODD : PF_FILL_NONZERO);
        // a clipped clip path (nested clips) is not supported by the d3d9 tiler either; the
        // upload rejects it
        path_clip_.push_back(clip.clip_path ? n_draw + *clip.clip_path : PF_NO_CLIP);
        path_is_clip_.push_back(1);
    }
    const RectF vb = scene->get_view_box();
    view_ = pf_scene_view{};
    view_.points = points_.data();
    view_.point_flags = flags_.data();
    view_.contour_start = contour_start_.data();
    view_.path_start = path_start_.data();
    view_.fill_rule = fill_rule_.data();
    view_.color = color_.data();
    view_.n_points = static_cast<uint32_t>(flags_.size());
    view_.n_contours = static_cast<uint32_t>(contour_start_.size() - 1);
    view_.n_paths = static_cast<uint32_t>(color_.size());
    if (!scene->clip_paths.empty()) {
        view_.path_clip = path_clip_.data();
        view_.path_is_clip = path_is_clip_.data();
    }
    // the view box with its origin (Scene::set_view_box); the image is the destination texture
    // (the tile pass covers it from (0, 0), core/d3d11/renderer.cpp:371, 443), or the view box's
    // lower-right corner when no destination is set
    view_box_[0] = vb.left;
    view_box_[1] = vb.top;
    view_box_[2] = vb.right;
    view_box_[3] = vb.bottom;
    view_.view_box = view_box_;
    const std::shared_ptr<Texture> dest = renderer ? renderer->get_dest_texture() : nullptr;
    if (dest) {
        view_.width = float(dest->get_size().x);
        view_.height = float(dest->get_size().y);
    } else {
        view_.width = vb.right > 1.0f ? vb.right : 1.0f;
        view_.height = vb.bottom > 1.0f ? vb.bottom : 1.0f;
    }
    view_.clear_color = 0;  // RendererD3D11::clear_color is transparent black (renderer.h:77)
    view_.load_action = PF_LOAD_CLEAR;
}

RendererCuda::RendererCuda(const std::shared_ptr<Device> &device, const std::shared_ptr<Queue> &queue,
                           int cuda_device)
    : Renderer(device, queue) {
    pf_config cfg{};
    cfg.device = cuda_device;
    if (pf_ctx_create(&cfg, &ctx_) != PF_OK) {
        Logger::error(std::string("RendererCuda: ") + pf_last_error(nullptr));
        ctx_ = nullptr;
    }
}

RendererCuda::~RendererCuda() {
    if (ctx_) pf_ctx_destroy(ctx_);
}

bool RendererCuda::load_sizer(const std::string &path) {
    learned_ = ctx_ && pf_sizer_load(ctx_, path.c_str()) == PF_OK;
    return learned_;
}

void RendererCuda::draw(const std::shared_ptr<SceneBuilder> &scene_builder, bool clear_dst_texture) {
    // errors are logged and the frame skipped, as the reference does (renderer.cpp:551-553)
    auto *builder = dynamic_cast<SceneBuilderCuda *>(scene_builder.get());
    if (!ctx_ || !builder) {
        Logger::error("RendererCuda: needs a SceneBuilderCuda and a CUDA context");
        return;
    }
    pf_scene_view view = builder->view();
    const size_t w = static_cast<size_t>(std::ceil(view.width)), h = static_cast<size_t>(std::ceil(view.height));
    // LOAD_ACTION_LOAD: composite over what this renderer last put into the destination
    const bool load = !clear_dst_texture && pixels_.size() == w * h * 4;
    view.load_action = load ? PF_LOAD_LOAD : PF_LOAD_CLEAR;
    int st = pf_scene_upload(ctx_, &view);
    if (st == PF_OK && load) st = pf_write_image(ctx_, 0, pixels_.data(), pixels_.size());
    // the library's default frame: with sizer weights it times the exact and the learned frame
    // on this scene and keeps the faster; without them it is the exact frame
    if (st == PF_OK) st = pf_render_auto(ctx_, 0, 1, &stats_);
    if (st == PF_OK) {
        pixels_.resize(w * h * 4);
        st = pf_read_image(ctx_, pixels_.data(), pixels_.size());
        if (st == PF_OK && dest_texture_) {
            auto encoder = device->create_command_encoder("RendererCuda upload");
            encoder->write_texture(dest_texture_, RectI({0, 0}, {int(w), int(h)}), pixels_.data());
            queue->submit(encoder, fence);
        }
    }
    if (st != PF_OK) Logger::error(std::string("RendererCuda: ") + pf_last_error(ctx_));
}

}  // namespace Pathfinder
