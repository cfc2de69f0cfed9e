// tx_dds.cu -- DDS container for compressed levels (host code only).
//
// The reference CLI writes and reads DDS files through the ddsfile crate
// (cli/src/main.rs:143-164, :167-196).  This is an independent implementation
// of the DDS layout (magic, 124-byte DDS_HEADER, 20-byte DDS_HEADER_DXT10)
// with the parameters the CLI passes: a DX10 header with the DXGI formats of
// format_to_dxgiformat (cli/src/main.rs:220-228), resource dimension
// Texture2D, array size 1, alpha mode premultiplied for BC1 and straight
// otherwise, a linear size of one level, and no mip count unless mips > 1.
// The reader accepts what the CLI's decompress_file accepts: a DX10 header
// with those DXGI formats and Texture2D, or a legacy DXT1/DXT3/DXT5 FourCC.
#include "texpresso_gb300.h"

#include <cstring>

namespace {

constexpr uint32_t kMagic = 0x20534444u;  // "DDS "
constexpr uint32_t kHeaderSize = 124, kPixelFormatSize = 32;
// DDS_HEADER flags
constexpr uint32_t DDSD_CAPS = 0x1, DDSD_HEIGHT = 0x2, DDSD_WIDTH = 0x4, DDSD_PIXELFORMAT = 0x1000,
                   DDSD_MIPMAPCOUNT = 0x20000, DDSD_LINEARSIZE = 0x80000;
constexpr uint32_t DDPF_FOURCC = 0x4;
constexpr uint32_t DDSCAPS_COMPLEX = 0x8, DDSCAPS_TEXTURE = 0x1000, DDSCAPS_MIPMAP = 0x400000;
constexpr uint32_t FOURCC_DX10 = 0x30315844u, FOURCC_DXT1 = 0x31545844u, FOURCC_DXT3 = 0x33545844u,
                   FOURCC_DXT5 = 0x35545844u;
constexpr uint32_t DIM_TEXTURE2D = 3;
constexpr uint32_t ALPHA_STRAIGHT = 1, ALPHA_PREMULTIPLIED = 2;
// DXGI_FORMAT values used by the CLI
constexpr uint32_t DXGI_BC1_UNORM_SRGB = 72, DXGI_BC2_UNORM_SRGB = 75, DXGI_BC3_UNORM_SRGB = 78,
                   DXGI_BC4_UNORM = 80, DXGI_BC5_UNORM = 83;

void put32(uint8_t *p, uint32_t v) {
    p[0] = (uint8_t)v; p[1] = (uint8_t)(v >> 8); p[2] = (uint8_t)(v >> 16); p[3] = (uint8_t)(v >> 24);
}
uint32_t get32(const uint8_t *p) {
    return (uint32_t)p[0] | ((uint32_t)p[1] << 8) | ((uint32_t)p[2] << 16) | ((uint32_t)p[3] << 24);
}

uint32_t dxgi_of(int format) {
    switch (format) {
    case TX_FORMAT_BC1: return DXGI_BC1_UNORM_SRGB;
    case TX_FORMAT_BC2: return DXGI_BC2_UNORM_SRGB;
    case TX_FORMAT_BC3: return DXGI_BC3_UNORM_SRGB;
    case TX_FORMAT_BC4: return DXGI_BC4_UNORM;
    case TX_FORMAT_BC5: return DXGI_BC5_UNORM;
    default: return 0;
    }
}

}  // namespace

extern "C" {

int tx_dds_write_header(int format, uint32_t width, uint32_t height, uint32_t mip_levels, uint8_t *out,
                        size_t out_len, size_t *written) {
    const uint32_t dxgi = dxgi_of(format);
    if (!dxgi) return TX_ERR_INVALID_FORMAT;
    if (width == 0 || height == 0 || mip_levels > 32) return TX_ERR_INVALID_ARGUMENT;
    if (!out || out_len < TX_DDS_HEADER_BYTES) return TX_ERR_OUTPUT_TOO_SMALL;
    uint8_t *h = out;
    std::memset(h, 0, TX_DDS_HEADER_BYTES);
    put32(h, kMagic);
    uint8_t *d = h + 4;
    uint32_t flags = DDSD_CAPS | DDSD_HEIGHT | DDSD_WIDTH | DDSD_PIXELFORMAT | DDSD_LINEARSIZE;
    uint32_t caps = DDSCAPS_TEXTURE;
    if (mip_levels > 1) {
        flags |= DDSD_MIPMAPCOUNT;
        caps |= DDSCAPS_COMPLEX | DDSCAPS_MIPMAP;
    }
    const uint64_t pitch = tx_num_blocks(width) * tx_block_size(format);
    const uint64_t linear = pitch * tx_num_blocks(height);
    if (linear > 0xFFFFFFFFull) return TX_ERR_INVALID_ARGUMENT;
    put32(d + 0, kHeaderSize);
    put32(d + 4, flags);
    put32(d + 8, height);
    put32(d + 12, width);
    put32(d + 16, (uint32_t)linear);  // dwPitchOrLinearSize
    put32(d + 20, 0);                 // dwDepth
    put32(d + 24, mip_levels > 1 ? mip_levels : 0);
    // dwReserved1[11] stay zero; DDS_PIXELFORMAT at offset 72
    put32(d + 72, kPixelFormatSize);
    put32(d + 76, DDPF_FOURCC);
    put32(d + 80, FOURCC_DX10);
    put32(d + 104, caps);             // dwCaps (dwCaps2..4, dwReserved2 zero)
    uint8_t *x = h + 4 + kHeaderSize;  // DDS_HEADER_DXT10
    put32(x + 0, dxgi);
    put32(x + 4, DIM_TEXTURE2D);
    put32(x + 8, 0);                   // miscFlag (not a cube map)
    put32(x + 12, 1);                  // arraySize
    put32(x + 16, format == TX_FORMAT_BC1 ? ALPHA_PREMULTIPLIED : ALPHA_STRAIGHT);
    if (written) *written = TX_DDS_HEADER_BYTES;
    return TX_OK;
}

int tx_dds_parse(const uint8_t *data, size_t len, int *format, uint32_t *width, uint32_t *height,
                 uint32_t *mip_levels, size_t *data_offset) {
    if (!data || len < 4 + kHeaderSize) return TX_ERR_INPUT_TOO_SMALL;
    if (get32(data) != kMagic) return TX_ERR_INVALID_ARGUMENT;
    const uint8_t *d = data + 4;
    if (get32(d) != kHeaderSize || get32(d + 72) != kPixelFormatSize) return TX_ERR_INVALID_ARGUMENT;
    const uint32_t h = get32(d + 8), w = get32(d + 12), flags = get32(d + 4);
    const uint32_t mips = (flags & DDSD_MIPMAPCOUNT) ? get32(d + 24) : 0;
    const uint32_t pf_flags = get32(d + 76), fourcc = get32(d + 80);
    int f = -1;
    size_t off = 4 + kHeaderSize;
    if ((pf_flags & DDPF_FOURCC) && fourcc == FOURCC_DX10) {
        if (len < off + 20) return TX_ERR_INPUT_TOO_SMALL;
        const uint8_t *x = data + off;
        if (get32(x + 4) != DIM_TEXTURE2D) return TX_ERR_INVALID_ARGUMENT;  // cli/src/main.rs:180-182
        switch (get32(x)) {
        case DXGI_BC1_UNORM_SRGB: f = TX_FORMAT_BC1; break;
        case DXGI_BC2_UNORM_SRGB: f = TX_FORMAT_BC2; break;
        case DXGI_BC3_UNORM_SRGB: f = TX_FORMAT_BC3; break;
        case DXGI_BC4_UNORM: f = TX_FORMAT_BC4; break;
        case DXGI_BC5_UNORM: f = TX_FORMAT_BC5; break;
        default: return TX_ERR_INVALID_FORMAT;  // cli/src/main.rs:230-239
        }
        off += 20;
    } else if (pf_flags & DDPF_FOURCC) {
        switch (fourcc) {
        case FOURCC_DXT1: f = TX_FORMAT_BC1; break;
        case FOURCC_DXT3: f = TX_FORMAT_BC2; break;
        case FOURCC_DXT5: f = TX_FORMAT_BC3; break;
        default: return TX_ERR_INVALID_FORMAT;  // cli/src/main.rs:241-248
        }
    } else {
        return TX_ERR_INVALID_FORMAT;
    }
    if (format) *format = f;
    if (width) *width = w;
    if (height) *height = h;
    if (mip_levels) *mip_levels = mips;
    if (data_offset) *data_offset = off;
    return TX_OK;
}

}  // extern "C"
