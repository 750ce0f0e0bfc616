// device_cuda.cpp - see device_cuda.h.
#include "device_cuda.h"

#include <cstring>

#include "common/logger.h"

namespace Pathfinder {

namespace {

// The objects a graphics device hands out that have nothing to do here: they only carry what
// the base classes hold.
class SamplerCuda : public Sampler {
public:
    explicit SamplerCuda(const SamplerDescriptor &d) : Sampler(d) {}
};

class DescriptorSetLayoutCuda : public DescriptorSetLayout {
public:
    explicit DescriptorSetLayoutCuda(const std::vector<DescriptorLayout> &l) : DescriptorSetLayout(l) {}
};

class DescriptorSetCuda : public DescriptorSet {
public:
    explicit DescriptorSetCuda(const std::shared_ptr<DescriptorSetLayout> &l) : DescriptorSet(l) {}
};

class RenderPassCuda : public RenderPass {
public:
    RenderPassCuda(AttachmentLoadOp op, const std::string &label) {
        load_op_ = op;
        label_ = label;
    }
};

class FramebufferCuda : public Framebuffer {
public:
    explicit FramebufferCuda(const std::shared_ptr<Texture> &t) : Framebuffer(t) {}
};

class ShaderModuleCuda : public ShaderModule {
public:
    explicit ShaderModuleCuda(const std::string &label) {
        label_ = label;
    }
};

class ComputePipelineCuda : public ComputePipeline {
public:
    ComputePipelineCuda(const std::shared_ptr<DescriptorSetLayout> &l, const std::string &label) {
        layout_ = l;
        label_ = label;
    }
};

class RenderPipelineCuda : public RenderPipeline {
public:
    RenderPipelineCuda(const std::vector<VertexInputAttributeDescription> &a, BlendState b,
                       const std::shared_ptr<DescriptorSetLayout> &l, const std::string &label)
        : RenderPipeline(a, b, label) {
        layout_ = l;
    }
};

// Copies a width x height region between a texture's rows and a packed buffer.
void copy_region(TextureCuda &t, uint32_t x0, uint32_t y0, uint32_t w, uint32_t h, uint8_t *packed, bool to_texture) {
    const size_t px = get_pixel_size(t.get_format());
    const size_t pitch = size_t(t.get_size().x) * px;
    for (uint32_t y = 0; y < h; y++) {
        uint8_t *row = t.pixels().data() + size_t(y0 + y) * pitch + size_t(x0) * px;
        uint8_t *p = packed + size_t(y) * w * px;
        if (to_texture) std::memcpy(row, p, size_t(w) * px);
        else std::memcpy(p, row, size_t(w) * px);
    }
}

}  // namespace

void BufferCuda::upload_via_mapping(size_t data_size, size_t offset, const void *data) {
    if (offset + data_size > bytes_.size()) {
        Logger::error("BufferCuda: write past the end of the buffer");
        return;
    }
    std::memcpy(bytes_.data() + offset, data, data_size);
}

void BufferCuda::download_via_mapping(size_t data_size, size_t offset, void *data) {
    if (offset + data_size > bytes_.size()) {
        Logger::error("BufferCuda: read past the end of the buffer");
        return;
    }
    std::memcpy(data, bytes_.data() + offset, data_size);
}

TextureCuda::TextureCuda(const TextureDescriptor &desc)
    : Texture(desc), pixels_(size_t(std::max(desc.size.x, 0)) * size_t(std::max(desc.size.y, 0)) *
                             get_pixel_size(desc.format)) {}

CommandEncoderCuda::CommandEncoderCuda(const std::shared_ptr<Device> &device, std::string label) {
    device_ = device;
    label_ = std::move(label);
}

std::shared_ptr<DeviceCuda> DeviceCuda::create(int cuda_device) {
    return std::shared_ptr<DeviceCuda>(new DeviceCuda(cuda_device));
}

std::shared_ptr<Framebuffer> DeviceCuda::create_framebuffer(const std::shared_ptr<RenderPass> &,
                                                            const std::shared_ptr<Texture> &texture,
                                                            const std::string &) {
    return std::make_shared<FramebufferCuda>(texture);
}

std::shared_ptr<Buffer> DeviceCuda::create_buffer(const BufferDescriptor &desc, const std::string &label) {
    auto b = std::make_shared<BufferCuda>(desc);
    b->set_label(label);
    return b;
}

std::shared_ptr<Texture> DeviceCuda::create_texture(const TextureDescriptor &desc, const std::string &label) {
    auto t = std::make_shared<TextureCuda>(desc);
    t->set_label(label);
    return t;
}

std::shared_ptr<Sampler> DeviceCuda::create_sampler(SamplerDescriptor descriptor) {
    return std::make_shared<SamplerCuda>(descriptor);
}

std::shared_ptr<CommandEncoder> DeviceCuda::create_command_encoder(const std::string &label) {
    return std::make_shared<CommandEncoderCuda>(shared_from_this(), label);
}

std::shared_ptr<DescriptorSetLayout> DeviceCuda::create_descriptor_set_layout(
    const std::vector<DescriptorLayout> &descriptors) {
    return std::make_shared<DescriptorSetLayoutCuda>(descriptors);
}

std::shared_ptr<DescriptorSet> DeviceCuda::create_descriptor_set(std::shared_ptr<DescriptorSetLayout> layout) {
    return std::make_shared<DescriptorSetCuda>(layout);
}

std::shared_ptr<RenderPass> DeviceCuda::create_render_pass(TextureFormat, AttachmentLoadOp load_op,
                                                           const std::string &label) {
    return std::make_shared<RenderPassCuda>(load_op, label);
}

std::shared_ptr<RenderPass> DeviceCuda::create_swap_chain_render_pass(TextureFormat, AttachmentLoadOp load_op) {
    return std::make_shared<RenderPassCuda>(load_op, "swap chain (headless: never presented)");
}

std::shared_ptr<ShaderModule> DeviceCuda::create_shader_module(const std::shared_ptr<Shader> &, const std::string &label) {
    return std::make_shared<ShaderModuleCuda>(label);
}

std::shared_ptr<ShaderModule> DeviceCuda::create_shader_module(const std::vector<char> &, ShaderStage,
                                                               const std::string &label) {
    return std::make_shared<ShaderModuleCuda>(label);
}

std::shared_ptr<RenderPipeline> DeviceCuda::create_render_pipeline(
    const std::shared_ptr<ShaderModule> &, const std::shared_ptr<ShaderModule> &,
    const std::vector<VertexInputAttributeDescription> &attribute_descriptions, BlendState blend_state,
    const std::shared_ptr<DescriptorSetLayout> &descriptor_set_layout, TextureFormat, const std::string &label) {
    return std::make_shared<RenderPipelineCuda>(attribute_descriptions, blend_state, descriptor_set_layout, label);
}

std::shared_ptr<ComputePipeline> DeviceCuda::create_compute_pipeline(
    const std::shared_ptr<ShaderModule> &, const std::shared_ptr<DescriptorSetLayout> &descriptor_set_layout,
    const std::string &label) {
    return std::make_shared<ComputePipelineCuda>(descriptor_set_layout, label);
}

std::shared_ptr<Fence> DeviceCuda::create_fence(const std::string &label) {
    auto f = std::make_shared<Fence>();
    f->label = label;
    return f;
}

void *DeviceCuda::map_staging(const StagingAllocation &allocation) {
    auto *b = dynamic_cast<BufferCuda *>(allocation.buffer.get());
    return b ? b->data() + allocation.offset : nullptr;
}

size_t DeviceCuda::get_aligned_uniform_size(size_t original_size) {
    return (original_size + 255) & ~size_t(255);
}

std::shared_ptr<Buffer> DeviceCuda::create_staging_buffer(size_t size) {
    return std::make_shared<BufferCuda>(BufferDescriptor{BufferType::Storage, size, MemoryProperty::HostVisibleAndCoherent});
}

void QueueCuda::submit(const std::shared_ptr<CommandEncoder> &encoder, const std::shared_ptr<Fence> &) {
    auto *enc = dynamic_cast<CommandEncoderCuda *>(encoder.get());
    if (!enc) {
        Logger::error("QueueCuda: the encoder does not come from a DeviceCuda");
        return;
    }
    for (const Command &cmd : enc->commands()) {
        switch (cmd.type) {
            case CommandType::WriteBuffer: {
                // the reference records reads with this type too (CommandEncoder::read_buffer);
                // a read's data pointer is set, a write's is not
                const auto &a = cmd.args.write_buffer;
                auto *dst = dynamic_cast<BufferCuda *>(a.buffer);
                auto *stg = dynamic_cast<BufferCuda *>(a.staging_buffer);
                if (!dst || !stg) break;
                if (cmd.args.read_buffer.data)
                    stg->upload_via_mapping(a.data_size, a.staging_offset, dst->data() + a.offset);
                else
                    dst->upload_via_mapping(a.data_size, a.offset, stg->data() + a.staging_offset);
                break;
            }
            case CommandType::ReadBuffer: {
                const auto &a = cmd.args.read_buffer;
                auto *src = dynamic_cast<BufferCuda *>(a.buffer);
                auto *stg = dynamic_cast<BufferCuda *>(a.staging_buffer);
                if (src && stg) stg->upload_via_mapping(a.data_size, a.staging_offset, src->data() + a.offset);
                break;
            }
            case CommandType::WriteTexture: {
                const auto &a = cmd.args.write_texture;
                auto *t = dynamic_cast<TextureCuda *>(a.texture);
                auto *stg = dynamic_cast<BufferCuda *>(a.staging_buffer);
                if (t && stg) copy_region(*t, a.offset_x, a.offset_y, a.width, a.height, stg->data() + a.staging_offset, true);
                break;
            }
            case CommandType::ReadTexture: {
                const auto &a = cmd.args.read_texture;
                auto *t = dynamic_cast<TextureCuda *>(a.texture);
                auto *stg = dynamic_cast<BufferCuda *>(a.staging_buffer);
                if (t && stg) copy_region(*t, a.offset_x, a.offset_y, a.width, a.height, stg->data() + a.staging_offset, false);
                break;
            }
            case CommandType::Draw:
            case CommandType::DrawIndexed:
            case CommandType::DrawInstanced:
            case CommandType::DrawIndirect:
            case CommandType::Dispatch:
            case CommandType::DispatchIndirect:
                skipped_++;
                Logger::error("QueueCuda: draws and dispatches have no shader pipeline here; skipped");
                break;
            default:
                break;  // pass and binding commands: nothing to do
        }
    }
    enc->finish();
}

}  // namespace Pathfinder
