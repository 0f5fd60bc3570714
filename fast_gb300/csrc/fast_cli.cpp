// `fast tau` and `fast alpha`: the command-line drop-in for the reference's
// tortuosity and reactive-area actions (fast/src/main.cpp,
// fast/src/TauModule.h:14-153, AlphaModule.h:8-233, VolumeIOModule.h:139-253,
// CSVOutputModule.h:35-112), over libfasttau.so's C ABI.
//
//   fast alpha <input.bin|tiff folder> [-d ...] [--basic] [crops] [-o out.csv]
//   fast slice <input.bin|tiff folder> [--size x[,y,z]] [--stride ..] [--begin ..]
//              [--end ..] [--out folder] [crops]
//
// alpha rows (AlphaModule::getAlpha, AlphaModule.h:28-179): without --basic,
// one row per direction with the area of the pore space connected to that
// face (rad; radTime = the labelling + tensor time / 6) and a DIR_NONE row
// with the whole solid/pore area; with --basic, one row per direction
// carrying the whole area (radBasic, radBasicTime) and no dir column.
// Columns are sorted by name as the reference's row map sorts them.  With
// --segmentinfo FILE the rows gain segmentVolumeRatio (volume fraction of the
// pore components not touching that face) and FILE gets one row per component
// not touching every face (getCCLSegmentInfo, VolumeSegmentation.cpp:135-215).
// --mesh FILE writes the surface of the volume zero-padded by one voxel as a
// Wavefront OBJ file (AlphaModule.h:150-173).
//
// slice rows (SliceModule.h:34-240): every sub-volume of --size at origins
// begin, begin + stride, ... with origin + size <= end (end defaults to the
// last voxel index, as the reference) is saved as <out>/<stem>/XXXX_YYYY_ZZZZ.bin
// and gets one row per positive direction in <out>/data.csv: ID (that path
// below <out>), alpha (the basic reactive area), porosity, tau (FP32 CG,
// tol 1e-5, 10000 iterations), sizex..z, originx..z, dir.  The reference
// solves the sub-volumes one at a time (small ones with its CPU solver);
// here all of them go through the batched GPU solver, up to 340 sub-volumes
// (1020 right-hand sides) per launch.
//
//   fast tau <input.bin|tiff folder> [-d x|y|z|xy..|all|pos|neg|xneg|yneg|zneg]
//            [--solver CG|BICGSTAB] [--tol N] [--iter N] [-p d|f|mixed]
//            [--sub x[,y,z]] [--origin x[,y,z]] [--randsub x[,y,z]]
//            [--aspect x,y,z] [-o out.csv] [-v] [--cpu] [-j N] [--over]
//
// For every direction one row is written (stdout, or appended to -o; the
// header goes first when the file is new), with the reference's columns in
// its order (a std::map of column names, so sorted): ID, device, dimx, dimy,
// dimz, dir, porosity, precision, tau, tauIter, tauNU, tauSolver, tauTime,
// tauTolerance.  As in the reference the porosity is computed once per
// volume, rounded to float and passed to every direction as precomputed, and
// tauTime covers one direction's getTortuosity call.  Every solve runs on the
// GPU: --cpu and -j are accepted for compatibility and change nothing
// (device is reported as GPU); --over has no counterpart.  -p mixed selects
// the engine's mixed-precision solver (precision column "mixed").  Input is a
// .bin volume (VolumeIO.cpp:279-305: int32 PrimitiveType, int32 x 3
// dimensions, one bool byte, raw x-fastest data) of type uchar, or a folder
// of 8-bit TIFF slices, which is read (fast_tiff_folder_read) and binarized
// with threshold 1.0 on the GPU (fast_binarize) as VolumeIOModule.h:57-63
// does.  .sph and .pos inputs (particle rasterisation) are not read.
#include <sys/stat.h>

#include <algorithm>
#include <array>
#include <cerrno>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <random>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

#include "fasttau.h"

namespace {

constexpr int32_t kTypeUchar = 2;  // PrimitiveType TYPE_UCHAR (PrimitiveTypes.h:11-24)

struct Vol {
    int64_t nx = 0, ny = 0, nz = 0;
    std::vector<uint8_t> data;  // x fastest
};

int usage(const char *why)
{
    if (why) std::cerr << "error: " << why << "\n";
    std::cerr << "usage: fast tau <input.bin|tiff folder> [-d x|y|z|all|pos|neg] [--solver CG|BICGSTAB] [--tol N]\n"
                 "                [--iter N] [-p d|f|mixed] [--sub x,y,z] [--origin x,y,z] [--randsub x,y,z]\n"
                 "                [--aspect x,y,z] [-o out.csv] [-v] [--cpu] [-j N]\n"
                 "       fast alpha <input.bin|tiff folder> [-d x|y|z|all|pos|neg] [--basic] [--sub x,y,z]\n"
                 "                [--origin x,y,z] [--randsub x,y,z] [--aspect x,y,z] [-o out.csv]\n"
                 "       fast slice <input.bin|tiff folder> [--size x,y,z] [--stride x,y,z] [--begin x,y,z]\n"
                 "                [--end x,y,z] [--out folder]\n";
    return why ? 1 : 0;
}

bool ends_with(const std::string &s, const std::string &ext)
{
    const size_t d = s.find_last_of('.');
    return d != std::string::npos && s.substr(d + 1) == ext;
}

// "x" or "x,y,z" (IVec3Reader / Vec3Reader, fast/src/utility.h:34-66).
template <typename T>
bool parse3(const std::string &v, T out[3])
{
    std::stringstream ss(v);
    std::string item;
    std::vector<std::string> parts;
    while (std::getline(ss, item, ',')) parts.push_back(item);
    try {
        if (parts.size() == 1) {
            out[0] = out[1] = out[2] = (T)std::stod(parts[0]);
        } else if (parts.size() == 3) {
            for (int k = 0; k < 3; k++) out[k] = (T)std::stod(parts[k]);
        } else {
            return false;
        }
    } catch (...) {
        return false;
    }
    return true;
}

// getDirs (fast/src/utility.h:77-109).
std::vector<int32_t> get_dirs(const std::string &f)
{
    if (f == "all") return {FAST_X_POS, FAST_X_NEG, FAST_Y_POS, FAST_Y_NEG, FAST_Z_POS, FAST_Z_NEG};
    if (f == "pos") return {FAST_X_POS, FAST_Y_POS, FAST_Z_POS};
    if (f == "neg") return {FAST_X_NEG, FAST_Y_NEG, FAST_Z_NEG};
    if (f == "xneg") return {FAST_X_NEG};
    if (f == "yneg") return {FAST_Y_NEG};
    if (f == "zneg") return {FAST_Z_NEG};
    std::vector<int32_t> d;
    for (char c : f) {
        if (c == 'x') d.push_back(FAST_X_POS);
        else if (c == 'y') d.push_back(FAST_Y_POS);
        else if (c == 'z') d.push_back(FAST_Z_POS);
    }
    if (d.empty()) d.push_back(FAST_X_POS);
    return d;
}

const char *dir_string(int32_t d)
{
    static const char *names[] = {"X_POS", "X_NEG", "Y_POS", "Y_NEG", "Z_POS", "Z_NEG"};
    return (d >= 0 && d < 6) ? names[d] : "DIR_NONE";
}

bool is_directory(const std::string &path)
{
    struct stat st;
    return stat(path.c_str(), &st) == 0 && S_ISDIR(st.st_mode);
}

// loadTiffFolder + binarize(1.0) (VolumeIOModule.h:57-63): the slices' raw
// values, then v < 255 -> 0, else 255, on the GPU.
bool load_tiff_folder(const std::string &path, Vol &v, std::string &err)
{
    if (fast_tiff_folder_info(path.c_str(), &v.nx, &v.ny, &v.nz) != FAST_OK) {
        err = fast_last_error();
        return false;
    }
    v.data.resize((size_t)(v.nx * v.ny * v.nz));
    if (fast_tiff_folder_read(path.c_str(), v.data.data(), v.data.size()) != FAST_OK ||
        fast_binarize(v.data.data(), v.data.size(), 1.0f) != FAST_OK) {
        err = fast_last_error();
        return false;
    }
    return true;
}

// loadVolumeBinary (fastlib/src/volume/VolumeIO.cpp:279-305).
bool load_bin(const std::string &path, Vol &v, std::string &err)
{
    std::ifstream f(path, std::ios::binary);
    if (!f.good()) {
        err = "Couldn't read file";
        return false;
    }
    int32_t type = 0, dim[3] = {0, 0, 0};
    char flag = 0;
    f.read((char *)&type, 4);
    f.read((char *)dim, 12);
    f.read(&flag, 1);
    if (!f.good()) {
        err = "truncated header";
        return false;
    }
    if (type != kTypeUchar) {
        err = "Mask must by type uchar";  // VolumeMeasures.cpp:50
        return false;
    }
    if (dim[0] <= 0 || dim[1] <= 0 || dim[2] <= 0) {
        err = "bad dimensions";
        return false;
    }
    v.nx = dim[0];
    v.ny = dim[1];
    v.nz = dim[2];
    v.data.resize((size_t)(v.nx * v.ny * v.nz));
    f.read((char *)v.data.data(), (std::streamsize)v.data.size());
    if ((size_t)f.gcount() != v.data.size()) {
        err = "truncated data";
        return false;
    }
    return true;
}

// Volume::resize(origin, size): keep the box [origin, origin + size).
Vol crop(const Vol &v, const int64_t o[3], const int64_t s[3])
{
    Vol r;
    r.nx = s[0];
    r.ny = s[1];
    r.nz = s[2];
    r.data.resize((size_t)(r.nx * r.ny * r.nz));
    for (int64_t z = 0; z < r.nz; z++)
        for (int64_t y = 0; y < r.ny; y++)
            memcpy(&r.data[(size_t)(r.nx * (y + r.ny * z))],
                   &v.data[(size_t)(o[0] + v.nx * (o[1] + y + v.ny * (o[2] + z)))], (size_t)r.nx);
    return r;
}

struct Row {
    std::string id, dir, precision, solver;
    int64_t dim[3];
    double porosity, tau, time, tol;
    int iter;
};

// CSVOutputModule::addRunRow (CSVOutputModule.h:35-89): header when the
// output is new (file absent, or the first row to stdout), appended rows.
void write_row(const std::string &out_path, bool &first_stdout, const Row &r)
{
    std::ostringstream line;
    line << r.id << "," << "GPU" << "," << r.dim[0] << "," << r.dim[1] << "," << r.dim[2] << "," << r.dir << ","
         << r.porosity << "," << r.precision << "," << r.tau << "," << r.iter << "," << 0 << "," << r.solver << ","
         << r.time << "," << r.tol << "\n";
    const char *header = "ID,device,dimx,dimy,dimz,dir,porosity,precision,tau,tauIter,tauNU,tauSolver,tauTime,"
                         "tauTolerance\n";
    if (out_path.empty()) {
        if (first_stdout) std::cout << header;
        first_stdout = false;
        std::cout << line.str();
        std::cout.flush();
        return;
    }
    bool is_new;
    {
        std::ifstream f(out_path);
        is_new = !f.is_open();
    }
    std::ofstream f(out_path, std::ios::app);
    if (is_new) f << header;
    f << line.str();
}

// CSVOutputModule::addRunRow for a row map: columns sorted by name, header
// when the output is new.
void write_map_row(const std::string &out_path, bool &first_stdout,
                   std::vector<std::pair<std::string, std::string>> row)
{
    std::sort(row.begin(), row.end());
    std::ostringstream header, line;
    for (size_t k = 0; k < row.size(); k++) {
        header << (k ? "," : "") << row[k].first;
        line << (k ? "," : "") << row[k].second;
    }
    header << "\n";
    line << "\n";
    if (out_path.empty()) {
        if (first_stdout) std::cout << header.str();
        first_stdout = false;
        std::cout << line.str();
        std::cout.flush();
        return;
    }
    bool is_new;
    {
        std::ifstream f(out_path);
        is_new = !f.is_open();
    }
    std::ofstream f(out_path, std::ios::app);
    if (is_new) f << header.str();
    f << line.str();
}

template <typename T>
std::string fmt(T v)
{
    std::ostringstream o;
    o << v;
    return o.str();
}

// One component of getCCLSegmentInfo (fastlib/src/volume/
// VolumeSegmentation.cpp:135-180): bounding box (max exclusive), voxel count,
// whether the box reaches a face.
struct SegInfo {
    int64_t minb[3], maxb[3];
    int64_t voxels = 0;
    bool at_boundary = false;
};

// getVolumeCCL(mask, 255) on the GPU, then getCCLSegmentInfo over the labels
// on the host, as the reference computes it (on retrieved labels).
bool segment_info(const Vol &vol, std::vector<SegInfo> &info, std::vector<uint8_t> &boundary, std::string &err)
{
    const size_t n = (size_t)(vol.nx * vol.ny * vol.nz);
    std::vector<uint32_t> labels(n);
    uint32_t k = 0;
    if (fast_ccl_label(vol.data.data(), vol.nx, vol.ny, vol.nz, 255, labels.data(), &k, nullptr, 0) != FAST_OK) {
        err = fast_last_error();
        return false;
    }
    boundary.assign((size_t)7 * k, 0);
    if (fast_ccl_label(vol.data.data(), vol.nx, vol.ny, vol.nz, 255, nullptr, &k, boundary.data(), boundary.size()) !=
        FAST_OK) {
        err = fast_last_error();
        return false;
    }
    const int64_t dim[3] = {vol.nx, vol.ny, vol.nz};
    info.assign(k, SegInfo{});
    for (SegInfo &g : info)
        for (int a = 0; a < 3; a++) {
            g.minb[a] = dim[a];
            g.maxb[a] = 0;
        }
    size_t i = 0;
    for (int64_t z = 0; z < vol.nz; z++)
        for (int64_t y = 0; y < vol.ny; y++)
            for (int64_t x = 0; x < vol.nx; x++, i++) {
                SegInfo &g = info[labels[i]];
                g.voxels++;
                const int64_t p[3] = {x, y, z};
                for (int a = 0; a < 3; a++) {
                    g.minb[a] = std::min(g.minb[a], p[a]);
                    g.maxb[a] = std::max(g.maxb[a], p[a]);
                }
            }
    for (SegInfo &g : info) {
        for (int a = 0; a < 3; a++) g.maxb[a] += 1;  // non-inclusive bounds
        g.at_boundary = g.maxb[0] == dim[0] || g.maxb[1] == dim[1] || g.maxb[2] == dim[2] || g.minb[0] == 0 ||
                        g.minb[1] == 0 || g.minb[2] == 0;
    }
    return true;
}

// getCCLSegmentRatio of filterSegmentInfo(info, ccl, dir) (VolumeSegmentation.
// cpp:182-215): the volume fraction of the components (label >= 1) that do
// not touch face `row` (row 6: not every face).
double segment_ratio(const std::vector<SegInfo> &info, const std::vector<uint8_t> &boundary, int row, int64_t n)
{
    const size_t k = info.size();
    int64_t vox = 0;
    for (size_t l = 1; l < k; l++)
        if (!boundary[(size_t)row * k + l]) vox += info[l].voxels;
    return (double)(float)((float)vox / (float)n);
}

// The --mesh export (AlphaModule.h:150-173): the volume zero-padded by one
// voxel (Volume::withZeroPadding), its surface triangles
// (fast_reactive_area_mesh), written as CUDA_VBO::saveObj does
// (fastlib/src/utility/DataPtr.cpp:684-740): vertices merged by exact
// position, their face normals summed and normalised, "v", "vn" and "f"
// lines.
int export_mesh(const Vol &vol, const std::string &path)
{
    Vol pad;
    pad.nx = vol.nx + 2;
    pad.ny = vol.ny + 2;
    pad.nz = vol.nz + 2;
    pad.data.assign((size_t)(pad.nx * pad.ny * pad.nz), 0);
    for (int64_t z = 0; z < vol.nz; z++)
        for (int64_t y = 0; y < vol.ny; y++)
            memcpy(&pad.data[(size_t)(1 + pad.nx * (y + 1 + pad.ny * (z + 1)))],
                   &vol.data[(size_t)(vol.nx * (y + vol.ny * z))], (size_t)vol.nx);
    uint64_t ntri = 0;
    if (fast_reactive_area_mesh(pad.data.data(), pad.nx, pad.ny, pad.nz, 0.5f, nullptr, 0, &ntri) != FAST_OK) {
        std::cerr << "error: " << fast_last_error() << "\n";
        return 1;
    }
    if (ntri == 0) {
        std::cerr << "Has no triangles" << std::endl;
        return 0;
    }
    std::vector<float> tri((size_t)ntri * 12);
    if (fast_reactive_area_mesh(pad.data.data(), pad.nx, pad.ny, pad.nz, 0.5f, tri.data(), ntri, &ntri) != FAST_OK) {
        std::cerr << "error: " << fast_last_error() << "\n";
        return 1;
    }
    std::cout << "Saving " << path << ", Vertices:" << ntri * 3 << std::endl;
    struct Key {
        uint32_t a, b, c;
        bool operator==(const Key &o) const { return a == o.a && b == o.b && c == o.c; }
    };
    struct KeyHash {
        size_t operator()(const Key &k) const { return ((size_t)k.a * 73856093u) ^ ((size_t)k.b * 19349663u) ^ ((size_t)k.c * 83492791u); }
    };
    std::unordered_map<Key, uint32_t, KeyHash> index;
    std::vector<std::array<float, 3>> verts, normals;
    std::vector<std::array<uint32_t, 3>> faces((size_t)ntri);
    for (uint64_t t = 0; t < ntri; t++) {
        const float *T = &tri[(size_t)t * 12];
        for (int q = 0; q < 3; q++) {
            Key k;
            memcpy(&k.a, &T[3 * q], 4);
            memcpy(&k.b, &T[3 * q + 1], 4);
            memcpy(&k.c, &T[3 * q + 2], 4);
            auto it = index.find(k);
            uint32_t id;
            if (it == index.end()) {
                id = (uint32_t)verts.size();
                verts.push_back({T[3 * q], T[3 * q + 1], T[3 * q + 2]});
                normals.push_back({T[9], T[10], T[11]});
                index.emplace(k, id);
            } else {
                id = it->second;
                for (int a = 0; a < 3; a++) normals[id][a] += T[9 + a];
            }
            faces[(size_t)t][q] = id;
        }
    }
    std::ofstream f(path);
    if (!f.good()) {
        std::cerr << "error: cannot write " << path << "\n";
        return 1;
    }
    for (const auto &v : verts) f << "v " << v[0] << " " << v[1] << " " << v[2] << "\n";
    for (auto n : normals) {
        const float l = std::sqrt(n[0] * n[0] + n[1] * n[1] + n[2] * n[2]);
        const float inv = l > 0.f ? 1.0f / l : 0.f;
        f << "vn " << n[0] * inv << " " << n[1] * inv << " " << n[2] * inv << "\n";
    }
    for (const auto &fc : faces) f << "f " << fc[0] + 1 << " " << fc[1] + 1 << " " << fc[2] + 1 << "\n";
    std::cout << "Done." << std::endl;
    return 0;
}

// AlphaModule::getAlpha (AlphaModule.h:28-179).
int run_alpha(const std::string &name, const Vol &vol, const std::vector<int32_t> &dirs, bool basic,
              const std::string &out_path, const std::string &info_path, const std::string &mesh_path)
{
    double phi = 0.0;
    if (fast_porosity(vol.data.data(), vol.nx, vol.ny, vol.nz, &phi, nullptr) != FAST_OK) {
        std::cerr << "error: " << fast_last_error() << "\n";
        return 1;
    }
    const std::vector<std::pair<std::string, std::string>> common = {
        {"ID", name}, {"dimx", fmt(vol.nx)}, {"dimy", fmt(vol.ny)}, {"dimz", fmt(vol.nz)},
        {"porosity", fmt((float)phi)}};
    bool first_stdout = true;
    auto timed_area = [&](double *area, double *secs) {
        const auto t0 = std::chrono::system_clock::now();
        const int st = fast_reactive_area(vol.data.data(), vol.nx, vol.ny, vol.nz, 0.5f, area);
        *secs = std::chrono::duration<double>(std::chrono::system_clock::now() - t0).count();
        return st;
    };
    if (!basic) {
        double tensor[6], solid = 0.0;
        const auto t0 = std::chrono::system_clock::now();
        int st = fast_reactive_area_tensor(vol.data.data(), vol.nx, vol.ny, vol.nz, 0.5f, tensor, &solid);
        const double rad_time = std::chrono::duration<double>(std::chrono::system_clock::now() - t0).count();
        if (st != FAST_OK) {
            std::cerr << "error: " << fast_last_error() << "\n";
            return 1;
        }
        std::vector<SegInfo> info;
        std::vector<uint8_t> boundary;
        const int64_t n = vol.nx * vol.ny * vol.nz;
        if (!info_path.empty()) {
            std::string err;
            if (!segment_info(vol, info, boundary, err)) {
                std::cerr << "error: " << err << "\n";
                return 1;
            }
        }
        for (int32_t d : dirs) {
            auto row = common;
            row.push_back({"rad", fmt(tensor[d])});
            row.push_back({"radTime", fmt(rad_time / 6.0f)});
            row.push_back({"dir", dir_string(d)});
            if (!info.empty()) row.push_back({"segmentVolumeRatio", fmt((float)segment_ratio(info, boundary, d, n))});
            write_map_row(out_path, first_stdout, row);
        }
        double area = 0.0, secs = 0.0;
        if ((st = timed_area(&area, &secs)) != FAST_OK) {
            std::cerr << "error: " << fast_last_error() << "\n";
            return 1;
        }
        auto row = common;
        row.push_back({"rad", fmt((float)area)});
        row.push_back({"radTime", fmt(secs)});
        row.push_back({"dir", "DIR_NONE"});
        if (!info.empty()) row.push_back({"segmentVolumeRatio", fmt((float)segment_ratio(info, boundary, 6, n))});
        write_map_row(out_path, first_stdout, row);
        // The components that do not touch every face (filterSegmentInfo with
        // DIR_NONE), one row each, to the segment-info CSV.
        bool info_first = true;
        const size_t k = info.size();
        for (size_t l = 1; l < k; l++) {
            if (boundary[6 * k + l]) continue;
            const SegInfo &g = info[l];
            write_map_row(info_path, info_first,
                          {{"ID", name}, {"minX", fmt(g.minb[0])}, {"minY", fmt(g.minb[1])}, {"minZ", fmt(g.minb[2])},
                           {"maxX", fmt(g.maxb[0])}, {"maxY", fmt(g.maxb[1])}, {"maxZ", fmt(g.maxb[2])},
                           {"labelID", fmt(l)}, {"voxelNum", fmt(g.voxels)}, {"atBoundary", fmt((int)g.at_boundary)}});
        }
    } else {
        double area = 0.0, secs = 0.0;
        if (timed_area(&area, &secs) != FAST_OK) {
            std::cerr << "error: " << fast_last_error() << "\n";
            return 1;
        }
        for (size_t k = 0; k < dirs.size(); k++) {
            auto row = common;
            row.push_back({"radBasic", fmt((float)area)});
            row.push_back({"radBasicTime", fmt(secs)});
            write_map_row(out_path, first_stdout, row);
        }
    }
    if (!mesh_path.empty()) return export_mesh(vol, mesh_path);
    return 0;
}

// mkdir -p
bool make_dirs(const std::string &path)
{
    std::string cur;
    std::stringstream ss(path);
    std::string part;
    if (!path.empty() && path[0] == '/') cur = "/";
    while (std::getline(ss, part, '/')) {
        if (part.empty()) continue;
        cur += part + "/";
        if (mkdir(cur.c_str(), 0755) != 0 && errno != EEXIST) return false;
    }
    return true;
}

// saveVolumeBinary (VolumeIO.cpp:256-277) of a uchar volume.
bool save_bin(const std::string &path, const Vol &v)
{
    std::ofstream f(path, std::ios::binary);
    if (!f.good()) return false;
    const int32_t type = kTypeUchar, dim[3] = {(int32_t)v.nx, (int32_t)v.ny, (int32_t)v.nz};
    const char flag = 0;
    f.write((const char *)&type, 4);
    f.write((const char *)dim, 12);
    f.write(&flag, 1);
    f.write((const char *)v.data.data(), (std::streamsize)v.data.size());
    return f.good();
}

// SliceModule::execute (SliceModule.h:34-240), without its PER_SLICE PNG
// branch (compiled out in the reference).
int run_slice(const std::string &name, const Vol &vol, const int64_t size[3], const int64_t stride[3],
              const int64_t begin_arg[3], const int64_t end_arg[3], const std::string &out_dir)
{
    const int64_t dim[3] = {vol.nx, vol.ny, vol.nz};
    int64_t begin[3], end[3];
    for (int k = 0; k < 3; k++) {
        begin[k] = std::min(begin_arg[k], dim[k] - 1);
        end[k] = std::max(end_arg[k], (int64_t)0);
        if (end[k] == 0) end[k] = dim[k] - 1;
        if (size[k] <= 0 || stride[k] <= 0) {
            std::cerr << "error: --size and --stride must be positive\n";
            return 1;
        }
    }
    // stem: the last component of the input name (explode on '/')
    std::string stem = name;
    {
        std::stringstream ss(name);
        std::string part;
        while (std::getline(ss, part, '/')) stem = part;
    }
    std::vector<std::array<int64_t, 3>> origins;
    for (int64_t x0 = begin[0]; x0 + size[0] <= end[0]; x0 += stride[0])
        for (int64_t y0 = begin[1]; y0 + size[1] <= end[1]; y0 += stride[1])
            for (int64_t z0 = begin[2]; z0 + size[2] <= end[2]; z0 += stride[2]) origins.push_back({x0, y0, z0});
    std::cout << "Subvolume count " << origins.size() << std::endl;
    if (origins.empty()) {
        std::cout << "Volume is not big enough " << dim[0] << ", " << dim[1] << ", " << dim[2] << ", need " << size[0]
                  << ", " << size[1] << ", " << size[2] << std::endl;
        return 0;
    }
    const std::string vol_dir = out_dir + "/" + stem;
    if (!make_dirs(vol_dir)) {
        std::cerr << "error: cannot create " << vol_dir << "\n";
        return 1;
    }
    const std::string csv = out_dir + "/data.csv";
    const int32_t dirs[3] = {FAST_X_POS, FAST_Y_POS, FAST_Z_POS};
    fast_tau_params p;
    fast_tau_params_init(&p);
    p.solver = FAST_SOLVER_CG;
    p.precision = FAST_PREC_F32;
    p.tolerance = std::pow(10.0, -5);
    p.max_iter = 10000;
    p.porosity = -1.0;  // each sub-volume's own (getPorosity, float)
    bool first_stdout = true;
    const size_t kChunk = 340;  // 3 right-hand sides each, within one launch's 1024
    for (size_t c0 = 0; c0 < origins.size(); c0 += kChunk) {
        const size_t c1 = std::min(origins.size(), c0 + kChunk);
        std::vector<Vol> subs(c1 - c0);
        std::vector<fast_tau_volume> tv;
        std::vector<double> alpha(c1 - c0), phi(c1 - c0);
        std::vector<std::string> ids(c1 - c0);
        for (size_t s = c0; s < c1; s++) {
            Vol &sv = subs[s - c0];
            sv = crop(vol, origins[s].data(), size);
            char buf[64];
            snprintf(buf, sizeof(buf), "%04lld_%04lld_%04lld.bin", (long long)origins[s][0], (long long)origins[s][1],
                     (long long)origins[s][2]);
            const std::string path = vol_dir + "/" + buf;
            ids[s - c0] = path.substr(out_dir.size() + 1);
            if (!save_bin(path, sv)) {
                std::cerr << "error: cannot write " << path << "\n";
                return 1;
            }
            // AlphaModule::getAlpha(subvolume, name, basic = true, {X_POS}):
            // porosity as float, radBasic as float.
            double ph = 0.0, area = 0.0;
            if (fast_porosity(sv.data.data(), sv.nx, sv.ny, sv.nz, &ph, nullptr) != FAST_OK ||
                fast_reactive_area(sv.data.data(), sv.nx, sv.ny, sv.nz, 0.5f, &area) != FAST_OK) {
                std::cerr << "error: " << fast_last_error() << "\n";
                return 1;
            }
            phi[s - c0] = ph;
            alpha[s - c0] = area;
            for (int32_t d : dirs) tv.push_back(fast_tau_volume{sv.data.data(), sv.nx, sv.ny, sv.nz, d, 0});
        }
        std::vector<fast_tau_result> res(tv.size());
        const int st = fast_tau_solve_batch(tv.data(), (int32_t)tv.size(), &p, res.data());
        if (st == FAST_CUDA_ERROR || st == FAST_NOMEM || st == FAST_TIMEOUT || st == FAST_BAD_ARG) {
            std::cerr << "error: " << fast_last_error() << "\n";
            return 1;
        }
        for (size_t s = c0; s < c1; s++) {
            for (int k = 0; k < 3; k++) {
                const fast_tau_result &r = res[(s - c0) * 3 + k];
                std::vector<std::pair<std::string, std::string>> row = {
                    {"ID", ids[s - c0]},
                    {"alpha", fmt((float)alpha[s - c0])},
                    {"porosity", fmt((float)phi[s - c0])},
                    {"tau", fmt(r.status == FAST_OK ? r.tau : 0.0)},
                    {"sizex", fmt(size[0])}, {"sizey", fmt(size[1])}, {"sizez", fmt(size[2])},
                    {"originx", fmt(origins[s][0])}, {"originy", fmt(origins[s][1])},
                    {"originz", fmt(origins[s][2])},
                    {"dir", dir_string(dirs[k])}};
                write_map_row(csv, first_stdout, row);
            }
        }
    }
    std::cout << "Generated " << origins.size() << " subvolumes" << std::endl;
    return 0;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 2) return usage("missing action");
    const std::string action = argv[1];
    if (action == "-h" || action == "--help") return usage(nullptr);
    if (action != "tau" && action != "alpha" && action != "slice")
        return usage("only the `tau`, `alpha` and `slice` actions are built");
    bool basic = false;
    int64_t slice_size[3] = {32, 32, 32}, slice_stride[3] = {1, 1, 1}, slice_begin[3] = {0, 0, 0},
            slice_end[3] = {0, 0, 0};
    std::string slice_out = "out";
    std::string info_path, mesh_path;

    std::string input, dir = "x-", solver = "CG", precision = "double", out_path;
    int tol_exp = 6;
    long long max_iter = 10000;
    bool verbose = false, has_sub = false, has_origin = false, has_rand = false, has_aspect = false;
    int64_t sub[3] = {0, 0, 0}, origin[3] = {0, 0, 0}, randsub[3] = {0, 0, 0};
    float aspect[3] = {1.f, 1.f, 1.f};
    for (int i = 2; i < argc; i++) {
        const std::string a = argv[i];
        auto next = [&](const char *what) -> std::string {
            if (i + 1 >= argc) {
                std::cerr << "error: " << what << " needs a value\n";
                std::exit(1);
            }
            return argv[++i];
        };
        if (a == "-h" || a == "--help") return usage(nullptr);
        else if (a == "-d" || a == "--dir") dir = next("-d");
        else if (a == "--solver") solver = next("--solver");
        else if (a == "--tol") tol_exp = std::atoi(next("--tol").c_str());
        else if (a == "--iter") max_iter = std::atoll(next("--iter").c_str());
        else if (a == "-p" || a == "--precision") precision = next("-p");
        else if (a == "-o" || a == "--output") out_path = next("-o");
        else if (a == "-v" || a == "--verbose") verbose = true;
        else if (a == "--cpu" || a == "--over" || a == "--oversubscribe") { /* accepted, no effect */ }
        else if (a == "--basic" && action == "alpha") basic = true;
        else if (a == "--size" && action == "slice") parse3(next("--size"), slice_size);
        else if (a == "--stride" && action == "slice") parse3(next("--stride"), slice_stride);
        else if (a == "--begin" && action == "slice") parse3(next("--begin"), slice_begin);
        else if (a == "--end" && action == "slice") parse3(next("--end"), slice_end);
        else if (a == "--out" && action == "slice") slice_out = next("--out");
        else if (a == "--segmentinfo" && action == "alpha") info_path = next("--segmentinfo");
        else if (a == "--mesh" && action == "alpha") mesh_path = next("--mesh");
        else if (a == "-j" || a == "--cputhreads") next("-j");
        else if (a == "--sub") has_sub = parse3(next("--sub"), sub);
        else if (a == "--origin") has_origin = parse3(next("--origin"), origin);
        else if (a == "--randsub") has_rand = parse3(next("--randsub"), randsub);
        else if (a == "--aspect") has_aspect = parse3(next("--aspect"), aspect);
        else if (!a.empty() && a[0] == '-') return usage(("unknown option " + a).c_str());
        else if (input.empty()) input = a;
        else return usage("more than one input");
    }
    if (input.empty()) return usage("Invalid input");

    Vol vol;
    std::string err;
    if (is_directory(input)) {
        if (!load_tiff_folder(input, vol, err)) {
            std::cerr << "Failed to load: " << err << "\n";
            return 1;
        }
    } else if (ends_with(input, "bin")) {
        if (!load_bin(input, vol, err)) {
            std::cerr << "Failed to load: " << err << "\n";
            return 1;
        }
    } else {
        return usage("input must be a .bin volume or a folder of TIFF slices");
    }
    // Crops (VolumeIOModule.h:180-248).
    if (has_sub || (has_origin && (origin[0] || origin[1] || origin[2]))) {
        const int64_t dim[3] = {vol.nx, vol.ny, vol.nz};
        int64_t lo[3], hi[3], size[3];
        for (int k = 0; k < 3; k++) {
            lo[k] = std::min(std::max(origin[k], (int64_t)0), dim[k]);
            hi[k] = std::min(std::max(origin[k] + sub[k], (int64_t)0), dim[k]);
            if (hi[k] <= lo[k]) {
                std::cerr << "error: Invalid resize options\n";
                return 1;
            }
            size[k] = hi[k] - lo[k];
        }
        vol = crop(vol, lo, size);
    } else if (has_rand) {
        const int64_t dim[3] = {vol.nx, vol.ny, vol.nz};
        std::mt19937_64 rng((uint64_t)std::chrono::system_clock::now().time_since_epoch().count());
        int64_t lo[3];
        for (int k = 0; k < 3; k++) {
            const int64_t room = dim[k] - randsub[k];
            if (randsub[k] <= 0 || room <= 0) {
                std::cerr << "error: Invalid resize options\n";
                return 1;
            }
            lo[k] = (int64_t)(rng() % (uint64_t)room);
        }
        vol = crop(vol, lo, randsub);
    }
    if (has_aspect) {
        int k = aspect[0] == 1.f ? 0 : (aspect[1] == 1.f ? 1 : (aspect[2] == 1.f ? 2 : -1));
        if (k < 0) {
            std::cerr << "error: Invalid aspect options, one dimension must equal to 1.0\n";
            return 1;
        }
        const int64_t dim[3] = {vol.nx, vol.ny, vol.nz};
        int64_t size[3];
        for (int a = 0; a < 3; a++) size[a] = std::min(std::max((int64_t)(dim[k] * aspect[a]), (int64_t)0), dim[a]);
        const int64_t lo[3] = {0, 0, 0};
        vol = crop(vol, lo, size);
    }

    if (action == "alpha") return run_alpha(input, vol, get_dirs(dir), basic, out_path, info_path, mesh_path);
    if (action == "slice") return run_slice(input, vol, slice_size, slice_stride, slice_begin, slice_end, slice_out);

    fast_tau_params p;
    fast_tau_params_init(&p);
    p.solver = solver == "BICGSTAB" ? FAST_SOLVER_BICGSTAB : FAST_SOLVER_CG;
    std::string prec_name = "double";
    if (precision == "float" || precision == "single" || precision == "f" || precision == "s") {
        p.precision = FAST_PREC_F32;
        prec_name = "single";
    } else if (precision == "mixed" || precision == "m") {
        p.precision = FAST_PREC_MIXED;
        prec_name = "mixed";
    } else {
        p.precision = FAST_PREC_F64;
    }
    p.tolerance = std::pow(10.0, -tol_exp);
    p.max_iter = (uint64_t)max_iter;
    p.verbose = verbose ? 1 : 0;

    double phi = 0.0;
    int st = fast_porosity(vol.data.data(), vol.nx, vol.ny, vol.nz, &phi, nullptr);
    if (st != FAST_OK) {
        std::cerr << "error: " << fast_last_error() << "\n";
        return 1;
    }
    // TauModule.h:68,80-81: float porosity, passed as precomputed.
    p.porosity = (double)(float)phi;

    bool first_stdout = true;
    int status = 0;
    for (int32_t d : get_dirs(dir)) {
        p.dir = d;
        if (verbose) std::cout << "Tau Direction " << d << std::endl;
        double tau = 0.0;
        uint64_t iters = 0;
        const auto t0 = std::chrono::system_clock::now();
        st = fast_tau_solve(vol.data.data(), vol.nx, vol.ny, vol.nz, &p, &tau, &iters, nullptr, nullptr);
        const std::chrono::duration<double> dt = std::chrono::system_clock::now() - t0;
        if (st != FAST_OK) {
            std::cerr << fast_last_error() << "\n";  // tau = 0, as the reference reports a failed solve
            if (st == FAST_CUDA_ERROR || st == FAST_NOMEM || st == FAST_TIMEOUT || st == FAST_BAD_ARG) status = 1;
        }
        if (verbose) std::cout << "Elapsed: " << dt.count() << "s (" << dt.count() / 60.0 << "m)" << std::endl;
        Row r{input, dir_string(d), prec_name, p.solver == FAST_SOLVER_BICGSTAB ? "BICGSTAB" : "CG",
              {vol.nx, vol.ny, vol.nz}, p.porosity, tau, dt.count(), p.tolerance, (int)iters};
        write_row(out_path, first_stdout, r);
    }
    return status;
}
