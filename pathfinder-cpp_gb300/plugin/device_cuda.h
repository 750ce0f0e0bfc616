// device_cuda.h - a headless Device / Queue for pathfinder-cpp on a CUDA-only host.
//
// The reference's Renderer base class needs a Device and a Queue (Renderer::Renderer,
// pathfinder/core/renderer.cpp:13-37: textures through the GPU memory allocator, a fence, a command
// encoder that writes the area LUT, a submit), and the palette uploads its metadata through them
// (Palette::build_paint_info, core/paint/palette.cpp:120-150).  Its devices are Vulkan, OpenGL and
// Metal (pathfinder/gpu/device.h:24-147), none of which exists on a compute-only GB300 host.
// DeviceCuda implements that interface without a graphics API, so that Canvas can construct
// RendererCuda there:
//
//  * buffers and textures are host memory (the CUDA renderer keeps its own device memory; what
//    the rest of the application reads from a texture - the destination image - is the pixels
//    the renderer wrote into it);
//  * command encoders record transfers as the base class does (write/read of buffers and
//    textures through staging buffers), and QueueCuda::submit carries them out in order, then
//    runs the encoder's callbacks;
//  * render and compute passes have nothing to run them (no shaders here): a submitted draw or
//    dispatch is logged as an error and skipped, as the reference logs and continues on errors.
//
// Compiled inside a pathfinder-cpp tree (it includes the reference's headers), next to
// renderer_cuda.h.
#pragma once

#include <memory>
#include <string>
#include <vector>

#include "gpu/device.h"
#include "gpu/queue.h"

namespace Pathfinder {

class BufferCuda : public Buffer {
public:
    explicit BufferCuda(const BufferDescriptor &desc) : Buffer(desc), bytes_(desc.size) {}

    void upload_via_mapping(size_t data_size, size_t offset, const void *data) override;
    void download_via_mapping(size_t data_size, size_t offset, void *data) override;

    uint8_t *data() {
        return bytes_.data();
    }

private:
    std::vector<uint8_t> bytes_;
};

class TextureCuda : public Texture {
public:
    explicit TextureCuda(const TextureDescriptor &desc);

    /// Row-major pixels, get_pixel_size(format) bytes each.
    std::vector<uint8_t> &pixels() {
        return pixels_;
    }

private:
    std::vector<uint8_t> pixels_;
};

class CommandEncoderCuda : public CommandEncoder {
public:
    explicit CommandEncoderCuda(const std::shared_ptr<Device> &device, std::string label);

    /// The recorded commands, for QueueCuda.
    const std::deque<Command> &commands() const {
        return commands_;
    }

    void finish() {
        submitted_ = true;
        invoke_callbacks();
    }

protected:
    bool prepare() override {
        prepared_ = true;
        return true;
    }
};

class DeviceCuda : public Device {
public:
    /// cuda_device: the CUDA device RendererCuda renders on (recorded for the application).
    static std::shared_ptr<DeviceCuda> create(int cuda_device = 0);

    int cuda_device() const {
        return cuda_device_;
    }

    std::shared_ptr<Framebuffer> create_framebuffer(const std::shared_ptr<RenderPass> &render_pass,
                                                    const std::shared_ptr<Texture> &texture,
                                                    const std::string &label) override;
    std::shared_ptr<Buffer> create_buffer(const BufferDescriptor &desc, const std::string &label) override;
    std::shared_ptr<Texture> create_texture(const TextureDescriptor &desc, const std::string &label) override;
    std::shared_ptr<Sampler> create_sampler(SamplerDescriptor descriptor) override;
    std::shared_ptr<CommandEncoder> create_command_encoder(const std::string &label) override;
    std::shared_ptr<DescriptorSetLayout> create_descriptor_set_layout(
        const std::vector<DescriptorLayout> &descriptors) override;
    std::shared_ptr<DescriptorSet> create_descriptor_set(std::shared_ptr<DescriptorSetLayout> layout) override;
    std::shared_ptr<RenderPass> create_render_pass(TextureFormat format,
                                                   AttachmentLoadOp load_op,
                                                   const std::string &label) override;
    std::shared_ptr<RenderPass> create_swap_chain_render_pass(TextureFormat format, AttachmentLoadOp load_op) override;
    std::shared_ptr<ShaderModule> create_shader_module(const std::shared_ptr<Shader> &shader,
                                                       const std::string &label) override;
    std::shared_ptr<ShaderModule> create_shader_module(const std::vector<char> &source_code,
                                                       ShaderStage shader_stage,
                                                       const std::string &label) override;
    std::shared_ptr<RenderPipeline> create_render_pipeline(
        const std::shared_ptr<ShaderModule> &vert_shader_module,
        const std::shared_ptr<ShaderModule> &frag_shader_module,
        const std::vector<VertexInputAttributeDescription> &attribute_descriptions,
        BlendState blend_state,
        const std::shared_ptr<DescriptorSetLayout> &descriptor_set_layout,
        TextureFormat target_format,
        const std::string &label) override;
    std::shared_ptr<ComputePipeline> create_compute_pipeline(
        const std::shared_ptr<ShaderModule> &comp_shader_module,
        const std::shared_ptr<DescriptorSetLayout> &descriptor_set_layout,
        const std::string &label) override;
    std::shared_ptr<Fence> create_fence(const std::string &label) override;

    void *map_staging(const StagingAllocation &allocation) override;
    size_t get_aligned_uniform_size(size_t original_size) override;

protected:
    std::shared_ptr<Buffer> create_staging_buffer(size_t size) override;

private:
    explicit DeviceCuda(int cuda_device) : Device(1), cuda_device_(cuda_device) {}

    int cuda_device_;
};

class QueueCuda : public Queue {
public:
    /// Carries out the encoder's transfers in order (host memory), then its callbacks.
    void submit(const std::shared_ptr<CommandEncoder> &encoder, const std::shared_ptr<Fence> &fence) override;

    /// Draws and dispatches submitted so far (skipped: nothing here runs shaders).
    size_t skipped_commands() const {
        return skipped_;
    }

private:
    size_t skipped_ = 0;
};

}  // namespace Pathfinder
