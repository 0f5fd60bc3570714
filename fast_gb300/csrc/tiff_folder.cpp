// TIFF-folder volumes: loadTiffFolder (fastlib/src/volume/VolumeIO.cpp:
// 197-254).  A folder of 2D slices, one per file, becomes a uint8 volume:
// nx, ny from the first slice in name order, nz = the number of *.tif and
// *.tiff files (VolumeIO.cpp:207-208), slice z at byte z*nx*ny.
//
// The reference reads each slice through TinyTIFF (an external submodule).
// This is a reader of baseline TIFF 6.0 of its own: both byte orders,
// uncompressed strips, 8 bits per sample, unsigned samples, chunky or planar
// samples of which sample 0 is taken, the first image (IFD) of each file.
// TinyTIFF reads the same subset; what it would mis-read (16-bit samples
// into an 8-bit buffer, slices of other sizes than the first) is rejected
// here with a message instead.
//
// Names follow the reference's rules: listDir sorts names byte-wise
// (VolumeIO.cpp:79-105) and checkExtension compares the text after the last
// '.' case-sensitively (VolumeIO.cpp:307-310).  Directories whose names end
// in .tif are skipped rather than counted.
#include <dirent.h>
#include <sys/stat.h>

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "fasttau.h"
#include "tau_errors.h"

namespace {

bool has_extension(const std::string &name, const char *ext)
{
    const size_t d = name.find_last_of('.');
    return name.substr(d == std::string::npos ? 0 : d + 1) == ext;
}

bool is_directory(const std::string &path)
{
    struct stat st;
    return stat(path.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

// Slice files of a folder, sorted byte-wise.
int list_slices(const char *folder, std::vector<std::string> &out)
{
    if (!folder) return ft_fail(FAST_BAD_ARG, "folder is NULL");
    DIR *d = opendir(folder);
    if (!d) return ft_fail(FAST_IO_ERROR, "Volume directory not found: %s", folder);
    while (dirent *e = readdir(d)) {
        const std::string name = e->d_name;
        if (!has_extension(name, "tiff") && !has_extension(name, "tif")) continue;
        if (is_directory(std::string(folder) + "/" + name)) continue;
        out.push_back(name);
    }
    closedir(d);
    std::sort(out.begin(), out.end());
    if (out.empty()) return ft_fail(FAST_IO_ERROR, "no .tif or .tiff files in %s", folder);
    return FAST_OK;
}

// One TIFF file held in memory.
struct Tiff {
    std::vector<uint8_t> bytes;
    bool big_endian = false;

    bool has(uint64_t off, uint64_t n) const { return off <= bytes.size() && n <= bytes.size() - off; }
    uint32_t u16(uint64_t off) const
    {
        const uint8_t *p = &bytes[off];
        return big_endian ? (uint32_t(p[0]) << 8 | p[1]) : (uint32_t(p[1]) << 8 | p[0]);
    }
    uint32_t u32(uint64_t off) const
    {
        const uint8_t *p = &bytes[off];
        return big_endian ? (uint32_t(p[0]) << 24 | uint32_t(p[1]) << 16 | uint32_t(p[2]) << 8 | p[3])
                          : (uint32_t(p[3]) << 24 | uint32_t(p[2]) << 16 | uint32_t(p[1]) << 8 | p[0]);
    }
};

// The first image of a file: the fields that locate sample 0 of each pixel.
struct Image {
    uint32_t width = 0, height = 0;
    uint32_t samples = 1;          // SamplesPerPixel (277)
    uint32_t compression = 1;      // Compression (259): 1 = none
    uint32_t planar = 1;           // PlanarConfiguration (284): 1 chunky, 2 planar
    uint32_t rows_per_strip = 0xFFFFFFFFu;
    std::vector<uint32_t> bits{1}; // BitsPerSample (258), one per sample; 1 when absent
    std::vector<uint32_t> format{1}; // SampleFormat (339): 1 = unsigned integer
    std::vector<uint32_t> strip_offsets, strip_counts;
    bool tiled = false;
};

// Integer values of one IFD entry (BYTE, SHORT or LONG).
bool entry_values(const Tiff &t, uint64_t entry, std::vector<uint32_t> &out)
{
    const uint32_t type = t.u16(entry + 2);
    const uint32_t count = t.u32(entry + 4);
    const uint32_t size = type == 1 ? 1 : type == 3 ? 2 : type == 4 ? 4 : 0;
    if (size == 0 || count == 0 || count > (1u << 28)) return false;
    const uint64_t total = (uint64_t)count * size;
    const uint64_t at = total <= 4 ? entry + 8 : t.u32(entry + 8);
    if (!t.has(at, total)) return false;
    out.resize(count);
    for (uint32_t k = 0; k < count; k++) {
        const uint64_t o = at + (uint64_t)k * size;
        out[k] = size == 1 ? t.bytes[o] : size == 2 ? t.u16(o) : t.u32(o);
    }
    return true;
}

int read_file(const std::string &path, Tiff &t)
{
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) return ft_fail(FAST_IO_ERROR, "Couldn't read tiff file %s", path.c_str());
    fseek(f, 0, SEEK_END);
    const long size = ftell(f);
    fseek(f, 0, SEEK_SET);
    t.bytes.resize(size > 0 ? (size_t)size : 0);
    const size_t got = t.bytes.empty() ? 0 : fread(t.bytes.data(), 1, t.bytes.size(), f);
    fclose(f);
    if (size <= 0 || got != t.bytes.size()) return ft_fail(FAST_IO_ERROR, "Couldn't read tiff file %s", path.c_str());
    t.big_endian = t.bytes.size() >= 2 && t.bytes[0] == 'M' && t.bytes[1] == 'M';
    return FAST_OK;
}

int parse_image(const std::string &path, const Tiff &t, Image &im)
{
    const bool ii = t.has(0, 8) && t.bytes[0] == 'I' && t.bytes[1] == 'I';
    const bool mm = t.has(0, 8) && t.bytes[0] == 'M' && t.bytes[1] == 'M';
    if (!ii && !mm) return ft_fail(FAST_IO_ERROR, "%s: not a TIFF file", path.c_str());
    const uint32_t magic = t.u16(2);
    if (magic == 43) return ft_fail(FAST_IO_ERROR, "%s: BigTIFF is not read", path.c_str());
    if (magic != 42) return ft_fail(FAST_IO_ERROR, "%s: not a TIFF file", path.c_str());
    const uint64_t ifd = t.u32(4);
    if (!t.has(ifd, 2)) return ft_fail(FAST_IO_ERROR, "%s: bad image directory offset", path.c_str());
    const uint32_t n = t.u16(ifd);
    if (!t.has(ifd + 2, (uint64_t)n * 12)) return ft_fail(FAST_IO_ERROR, "%s: truncated image directory", path.c_str());
    std::vector<uint32_t> v;
    for (uint32_t k = 0; k < n; k++) {
        const uint64_t e = ifd + 2 + (uint64_t)k * 12;
        const uint32_t tag = t.u16(e);
        switch (tag) {
        case 256: case 257: case 259: case 277: case 278: case 284:
            if (!entry_values(t, e, v)) return ft_fail(FAST_IO_ERROR, "%s: bad field %u", path.c_str(), tag);
            if (tag == 256) im.width = v[0];
            if (tag == 257) im.height = v[0];
            if (tag == 259) im.compression = v[0];
            if (tag == 277) im.samples = v[0];
            if (tag == 278) im.rows_per_strip = v[0];
            if (tag == 284) im.planar = v[0];
            break;
        case 258: case 339: case 273: case 279:
            if (!entry_values(t, e, v)) return ft_fail(FAST_IO_ERROR, "%s: bad field %u", path.c_str(), tag);
            if (tag == 258) im.bits = v;
            if (tag == 339) im.format = v;
            if (tag == 273) im.strip_offsets = v;
            if (tag == 279) im.strip_counts = v;
            break;
        case 322: case 323: case 324: case 325:
            im.tiled = true;
            break;
        default:
            break;
        }
    }
    if (im.width == 0 || im.height == 0) return ft_fail(FAST_IO_ERROR, "%s: no image size", path.c_str());
    if (im.samples == 0) return ft_fail(FAST_IO_ERROR, "%s: zero samples per pixel", path.c_str());
    for (uint32_t s = 0; s < im.samples; s++) {
        const uint32_t bits = im.bits[std::min<size_t>(s, im.bits.size() - 1)];
        const uint32_t fmt = im.format[std::min<size_t>(s, im.format.size() - 1)];
        if (bits != 8 || fmt != 1)
            return ft_fail(FAST_BAD_TYPE, "%s: only uint8 supported right now (%u bits, sample format %u)",
                           path.c_str(), bits, fmt);
    }
    if (im.compression != 1)
        return ft_fail(FAST_IO_ERROR, "%s: compressed TIFF (compression %u) is not read", path.c_str(), im.compression);
    if (im.tiled || im.strip_offsets.empty()) return ft_fail(FAST_IO_ERROR, "%s: tiled TIFF is not read", path.c_str());
    if (im.planar != 1 && im.planar != 2)
        return ft_fail(FAST_IO_ERROR, "%s: bad planar configuration %u", path.c_str(), im.planar);
    if (im.rows_per_strip == 0) im.rows_per_strip = 0xFFFFFFFFu;
    return FAST_OK;
}

// Sample 0 of every pixel, rows in order, x fastest, into out[width*height].
int read_sample0(const std::string &path, const Tiff &t, const Image &im, uint8_t *out)
{
    const uint64_t rps = std::min<uint64_t>(im.rows_per_strip, im.height);
    const uint64_t strips_per_plane = (im.height + rps - 1) / rps;
    const uint64_t step = im.planar == 1 ? im.samples : 1;  // bytes between pixels
    const uint64_t row_bytes = (uint64_t)im.width * step;
    if (im.strip_offsets.size() < strips_per_plane)
        return ft_fail(FAST_IO_ERROR, "%s: %zu strips, %llu needed", path.c_str(), im.strip_offsets.size(),
                       (unsigned long long)strips_per_plane);
    for (uint64_t y = 0; y < im.height; y++) {
        const uint64_t s = y / rps;
        const uint64_t within = (y - s * rps) * row_bytes;
        if (s < im.strip_counts.size() && within + row_bytes > im.strip_counts[s])
            return ft_fail(FAST_IO_ERROR, "%s: strip %llu is too short", path.c_str(), (unsigned long long)s);
        const uint64_t at = (uint64_t)im.strip_offsets[s] + within;
        if (!t.has(at, row_bytes)) return ft_fail(FAST_IO_ERROR, "%s: truncated image data", path.c_str());
        const uint8_t *src = &t.bytes[at];
        uint8_t *dst = out + y * im.width;
        if (step == 1) {
            memcpy(dst, src, im.width);
        } else {
            for (uint64_t x = 0; x < im.width; x++) dst[x] = src[x * step];
        }
    }
    return FAST_OK;
}

int slice_header(const std::string &path, Tiff &t, Image &im)
{
    int s = read_file(path, t);
    if (s != FAST_OK) return s;
    return parse_image(path, t, im);
}

}  // namespace

extern "C" {

FAST_API int fast_tiff_folder_info(const char *folder, int64_t *nx, int64_t *ny, int64_t *nz)
{
    ft_clear_error();
    if (!nx || !ny || !nz) return ft_fail(FAST_BAD_ARG, "null dimension pointer");
    std::vector<std::string> names;
    int s = list_slices(folder, names);
    if (s != FAST_OK) return s;
    Tiff t;
    Image im;
    s = slice_header(std::string(folder) + "/" + names[0], t, im);
    if (s != FAST_OK) return s;
    *nx = im.width;
    *ny = im.height;
    *nz = (int64_t)names.size();
    return FAST_OK;
}

FAST_API int fast_tiff_folder_read(const char *folder, uint8_t *out, uint64_t capacity)
{
    ft_clear_error();
    if (!out) return ft_fail(FAST_NO_HOST_DATA, "output buffer is NULL");
    std::vector<std::string> names;
    int s = list_slices(folder, names);
    if (s != FAST_OK) return s;
    uint64_t nx = 0, ny = 0;
    for (size_t z = 0; z < names.size(); z++) {
        const std::string path = std::string(folder) + "/" + names[z];
        Tiff t;
        Image im;
        s = slice_header(path, t, im);
        if (s != FAST_OK) return s;
        if (z == 0) {
            nx = im.width;
            ny = im.height;
            if (nx * ny * names.size() > capacity)
                return ft_fail(FAST_BAD_ARG, "buffer holds %llu bytes, %llu needed", (unsigned long long)capacity,
                               (unsigned long long)(nx * ny * names.size()));
        } else if (im.width != nx || im.height != ny) {
            return ft_fail(FAST_IO_ERROR, "%s is %ux%u, the first slice is %llux%llu", path.c_str(), im.width,
                           im.height, (unsigned long long)nx, (unsigned long long)ny);
        }
        s = read_sample0(path, t, im, out + z * nx * ny);
        if (s != FAST_OK) return s;
    }
    return FAST_OK;
}

}  // extern "C"
