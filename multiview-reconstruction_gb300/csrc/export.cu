// Export of the deconvolved volume (the step after the iteration: Image_Deconvolution's
// ImgExport, MV/export/*.java of the reference):
//   mvr_export_tiff  Save3dTIFF.exportImage / saveTiffStack (MV/export/Save3dTIFF.java:86-160):
//                    one ImageJ stack of 32-bit float slices with the calibration and the
//                    display range 0..255 that DisplayImage.getImagePlusInstance sets
//   mvr_export_n5    ExportN5Api with the N5 format and no compression (MV/export/ExportN5Api.java):
//                    a float32 dataset of raw blocks, one file per grid position
// The volume may be in host or device memory (device volumes are read back in slabs through
// one host buffer).  The writers are host code: file formats, no GPU work.
#include <cuda_runtime.h>

#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/mvr_gb300.h"

namespace {

void put_error(char *err, int len, const std::string &msg)
{
    if (err && len > 0) std::snprintf(err, (size_t)len, "%s", msg.c_str());
}

void be16(std::vector<uint8_t> &b, uint16_t v)
{
    b.push_back((uint8_t)(v >> 8));
    b.push_back((uint8_t)v);
}
void be32(std::vector<uint8_t> &b, uint32_t v)
{
    for (int s = 24; s >= 0; s -= 8) b.push_back((uint8_t)(v >> s));
}
void put_be32(uint8_t *p, uint32_t v)
{
    for (int i = 0; i < 4; ++i) p[i] = (uint8_t)(v >> (24 - 8 * i));
}

// Big-endian IEEE floats of n values (TIFF "MM" and N5 blocks are big-endian).
void floats_be(const float *src, size_t n, uint8_t *dst)
{
    for (size_t i = 0; i < n; ++i) {
        uint32_t u;
        std::memcpy(&u, src + i, 4);
        put_be32(dst + 4 * i, u);
    }
}

// Reads z-slabs of the volume into host memory (a device volume through `stage`).
struct SlabReader {
    const float *vol;
    bool dev;
    long long plane;
    std::vector<float> stage;
    const float *slab(long long z0, long long nz, std::string &e)
    {
        if (!dev) return vol + z0 * plane;
        stage.resize((size_t)(nz * plane));
        const cudaError_t c =
            cudaMemcpy(stage.data(), vol + z0 * plane, sizeof(float) * (size_t)(nz * plane), cudaMemcpyDeviceToHost);
        if (c != cudaSuccess) {
            e = cudaGetErrorString(c);
            return nullptr;
        }
        return stage.data();
    }
};

struct Tag {
    uint16_t id, type;
    uint32_t count, value;  // value or offset
};

// One IFD: entries sorted by tag id, the offset of the next IFD.
void write_ifd(std::vector<uint8_t> &b, std::vector<Tag> tags, uint32_t next)
{
    be16(b, (uint16_t)tags.size());
    for (const Tag &t : tags) {
        be16(b, t.id);
        be16(b, t.type);
        be32(b, t.count);
        if (t.type == 3 && t.count == 1) {  // SHORT: left-justified in the value field
            be16(b, (uint16_t)t.value);
            be16(b, 0);
        } else {
            be32(b, t.value);
        }
    }
    be32(b, next);
}

bool mkdir_p(const std::string &path)
{
    std::string cur;
    size_t i = 0;
    while (i <= path.size()) {
        const size_t j = path.find('/', i);
        cur = path.substr(0, j == std::string::npos ? path.size() : j);
        if (!cur.empty() && mkdir(cur.c_str(), 0777) != 0 && errno != EEXIST) return false;
        if (j == std::string::npos) break;
        i = j + 1;
    }
    return true;
}

}  // namespace

extern "C" int mvr_export_tiff(const char *path, const float *volume, const long long dims[3], int on_device,
                               const double calibration[3], const char *unit, char *err, int err_len)
{
    if (!path || !volume || !dims) {
        put_error(err, err_len, "path, volume and dims must not be NULL");
        return MVR_ERR_ARG;
    }
    const long long W = dims[0], H = dims[1], Z = dims[2];
    if (W < 1 || H < 1 || Z < 1 || W > 65535 || H > 65535) {
        put_error(err, err_len, "dims must be >= 1 (width and height <= 65535)");
        return MVR_ERR_ARG;
    }
    const double cal[3] = {calibration ? calibration[0] : 1.0, calibration ? calibration[1] : 1.0,
                           calibration ? calibration[2] : 1.0};
    const long long slice = W * H * 4;
    // layout: header, IFD 0, description, resolutions, pixel data, IFDs 1..Z-1
    char desc[512];
    std::snprintf(desc, sizeof(desc), "ImageJ=1.54f\nimages=%lld\nslices=%lld\nunit=%s\nspacing=%.17g\nloop=false\n"
                                      "min=0.0\nmax=255.0\n",
                  Z, Z, (unit && unit[0]) ? unit : "px", cal[2]);
    const uint32_t ndesc = (uint32_t)std::strlen(desc) + 1;
    const int ntags0 = 15, ntags = 14;
    const uint64_t ifd0 = 8, ifd0_len = 2 + 12 * ntags0 + 4;
    const uint64_t desc_off = ifd0 + ifd0_len;
    const uint64_t res_off = desc_off + ndesc + (ndesc & 1);
    const uint64_t data_off = res_off + 16;
    const uint64_t ifd_len = 2 + 12 * ntags + 4;
    const uint64_t tail = data_off + (uint64_t)slice * Z;
    if (tail + ifd_len * (uint64_t)(Z - 1) > 0xFFFFFFFFull) {
        put_error(err, err_len, "the stack exceeds the 4 GB offsets of a TIFF file");
        return MVR_ERR_UNSUPPORTED;
    }
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        put_error(err, err_len, std::string("cannot open ") + path + ": " + std::strerror(errno));
        return MVR_ERR_ARG;
    }
    auto fail_io = [&](const std::string &m) {
        std::fclose(f);
        put_error(err, err_len, m);
        return MVR_ERR_ARG;
    };
    const uint32_t xres_num = (uint32_t)std::lround(1e6 / cal[0]), yres_num = (uint32_t)std::lround(1e6 / cal[1]);
    auto tags_for = [&](uint64_t strip, bool first) {
        std::vector<Tag> t;
        t.push_back({254, 4, 1, 0});                               // NewSubfileType
        t.push_back({256, 4, 1, (uint32_t)W});                     // ImageWidth
        t.push_back({257, 4, 1, (uint32_t)H});                     // ImageLength
        t.push_back({258, 3, 1, 32});                              // BitsPerSample
        t.push_back({259, 3, 1, 1});                               // Compression: none
        t.push_back({262, 3, 1, 1});                               // Photometric: black is zero
        if (first) t.push_back({270, 2, ndesc, (uint32_t)desc_off});  // ImageDescription
        t.push_back({273, 4, 1, (uint32_t)strip});                 // StripOffsets
        t.push_back({277, 3, 1, 1});                               // SamplesPerPixel
        t.push_back({278, 4, 1, (uint32_t)H});                     // RowsPerStrip
        t.push_back({279, 4, 1, (uint32_t)slice});                 // StripByteCounts
        t.push_back({282, 5, 1, (uint32_t)res_off});               // XResolution
        t.push_back({283, 5, 1, (uint32_t)(res_off + 8)});         // YResolution
        t.push_back({296, 3, 1, 1});                               // ResolutionUnit: none
        t.push_back({339, 3, 1, 3});                               // SampleFormat: IEEE float
        return t;
    };
    std::vector<uint8_t> head = {'M', 'M', 0, 42};
    be32(head, (uint32_t)ifd0);
    write_ifd(head, tags_for(data_off, true), Z > 1 ? (uint32_t)tail : 0);
    head.insert(head.end(), desc, desc + ndesc);
    if (ndesc & 1) head.push_back(0);
    be32(head, xres_num);
    be32(head, 1000000);
    be32(head, yres_num);
    be32(head, 1000000);
    if (head.size() != data_off) return fail_io("TIFF layout error");
    if (std::fwrite(head.data(), 1, head.size(), f) != head.size()) return fail_io("write failed");
    SlabReader rd{volume, on_device != 0, W * H, {}};
    const long long zs = std::max<long long>(1, (64ll << 20) / slice);
    std::vector<uint8_t> buf;
    for (long long z0 = 0; z0 < Z; z0 += zs) {
        const long long nz = std::min(zs, Z - z0);
        std::string e;
        const float *p = rd.slab(z0, nz, e);
        if (!p) return fail_io("reading the device volume: " + e);
        buf.resize((size_t)(nz * slice));
        floats_be(p, (size_t)(nz * W * H), buf.data());
        if (std::fwrite(buf.data(), 1, buf.size(), f) != buf.size()) return fail_io("write failed");
    }
    std::vector<uint8_t> ifds;
    for (long long z = 1; z < Z; ++z) {
        const uint64_t next = z + 1 < Z ? tail + ifd_len * (uint64_t)z : 0;
        write_ifd(ifds, tags_for(data_off + (uint64_t)slice * z, false), (uint32_t)next);
    }
    if (!ifds.empty() && std::fwrite(ifds.data(), 1, ifds.size(), f) != ifds.size()) return fail_io("write failed");
    if (std::fclose(f) != 0) {
        put_error(err, err_len, "close failed");
        return MVR_ERR_ARG;
    }
    return MVR_OK;
}

extern "C" int mvr_export_n5(const char *root, const char *dataset, const float *volume, const long long dims[3],
                             int on_device, const int block_size[3], char *err, int err_len)
{
    if (!root || !dataset || !volume || !dims || !block_size) {
        put_error(err, err_len, "root, dataset, volume, dims and block_size must not be NULL");
        return MVR_ERR_ARG;
    }
    for (int d = 0; d < 3; ++d)
        if (dims[d] < 1 || block_size[d] < 1) {
            put_error(err, err_len, "dims and block sizes must be >= 1");
            return MVR_ERR_ARG;
        }
    const std::string dir = std::string(root) + "/" + dataset;
    if (!mkdir_p(dir)) {
        put_error(err, err_len, "cannot create " + dir + ": " + std::strerror(errno));
        return MVR_ERR_ARG;
    }
    auto write_text = [&](const std::string &p, const std::string &s) {
        FILE *f = std::fopen(p.c_str(), "wb");
        if (!f) return false;
        const bool ok = std::fwrite(s.data(), 1, s.size(), f) == s.size();
        return std::fclose(f) == 0 && ok;
    };
    if (!write_text(std::string(root) + "/attributes.json", "{\"n5\":\"4.0.0\"}")) {
        put_error(err, err_len, std::string("cannot write ") + root + "/attributes.json");
        return MVR_ERR_ARG;
    }
    char attr[512];
    std::snprintf(attr, sizeof(attr),
                  "{\"dimensions\":[%lld,%lld,%lld],\"blockSize\":[%d,%d,%d],\"dataType\":\"float32\","
                  "\"compression\":{\"type\":\"raw\"}}",
                  dims[0], dims[1], dims[2], block_size[0], block_size[1], block_size[2]);
    if (!write_text(dir + "/attributes.json", attr)) {
        put_error(err, err_len, "cannot write " + dir + "/attributes.json");
        return MVR_ERR_ARG;
    }
    const long long X = dims[0], Y = dims[1], Z = dims[2];
    SlabReader rd{volume, on_device != 0, X * Y, {}};
    std::vector<float> blk;
    std::vector<uint8_t> out;
    for (long long bz = 0; bz * block_size[2] < Z; ++bz) {
        const long long z0 = bz * block_size[2], nz = std::min<long long>(block_size[2], Z - z0);
        std::string e;
        const float *slab = rd.slab(z0, nz, e);
        if (!slab) {
            put_error(err, err_len, "reading the device volume: " + e);
            return MVR_ERR_CUDA;
        }
        for (long long by = 0; by * block_size[1] < Y; ++by)
            for (long long bx = 0; bx * block_size[0] < X; ++bx) {
                const long long y0 = by * block_size[1], x0 = bx * block_size[0];
                const long long ny = std::min<long long>(block_size[1], Y - y0), nx = std::min<long long>(block_size[0], X - x0);
                blk.resize((size_t)(nx * ny * nz));
                for (long long z = 0; z < nz; ++z)
                    for (long long y = 0; y < ny; ++y)
                        std::memcpy(&blk[(size_t)((z * ny + y) * nx)], slab + (z * Y + y0 + y) * X + x0,
                                    sizeof(float) * (size_t)nx);
                // N5 block: mode 0, number of dimensions, the block's size per dimension
                // (clipped at the border), then the values, all big-endian
                out.clear();
                be16(out, 0);
                be16(out, 3);
                be32(out, (uint32_t)nx);
                be32(out, (uint32_t)ny);
                be32(out, (uint32_t)nz);
                const size_t h = out.size();
                out.resize(h + 4 * blk.size());
                floats_be(blk.data(), blk.size(), out.data() + h);
                const std::string bdir = dir + "/" + std::to_string(bx) + "/" + std::to_string(by);
                if (!mkdir_p(bdir)) {
                    put_error(err, err_len, "cannot create " + bdir);
                    return MVR_ERR_ARG;
                }
                const std::string bpath = bdir + "/" + std::to_string(bz);
                FILE *f = std::fopen(bpath.c_str(), "wb");
                if (!f) {
                    put_error(err, err_len, "cannot write " + bpath);
                    return MVR_ERR_ARG;
                }
                const bool ok = std::fwrite(out.data(), 1, out.size(), f) == out.size();
                if (std::fclose(f) != 0 || !ok) {
                    put_error(err, err_len, "write failed: " + bpath);
                    return MVR_ERR_ARG;
                }
            }
    }
    return MVR_OK;
}
