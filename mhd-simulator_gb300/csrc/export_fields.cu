// export_fields.cu -- accepted fluid fields written as a frame directory: the
// reference's headless export format (RunState::export_fields,
// src/run/export.rs:9-60; docs/RUNS.md:87-88).
//
// The directory is created exclusively (an existing one is never touched),
// fluid.bin holds the cell records exactly as they sit in device memory
// (16 f32 per cell, x fastest, then y, then z; host byte order), and
// metadata.json is published last by renaming metadata.writing, so an
// incomplete export has no metadata.  On any failure the directory this call
// created is removed again.
#include <cuda_runtime.h>
#include <sys/stat.h>

#include <cerrno>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <filesystem>
#include <string>
#include <vector>

#include "../../include/mhdproj.h"

namespace mhdproj {
void set_global_error(const std::string& msg);
}

namespace {

std::string json_number(double v) {
    if (!std::isfinite(v)) return "null";
    char buf[64];
    snprintf(buf, sizeof buf, "%.17g", v);
    return buf;
}

int export_error(const std::string& msg) {
    mhdproj::set_global_error(msg);
    return MHDPROJ_ERR_INVALID;
}

}  // namespace

extern "C" int mhdproj_export_fields(const mhdproj_grid* grid, const float* cells, const char* directory,
                                     uint64_t step, double time_s, const float origin_m[3], int moving_interface,
                                     const char* forcing_kind) {
    namespace fs = std::filesystem;
    if (!grid || !cells || !directory || !directory[0]) return export_error("grid, cells and directory are required");
    const uint64_t n = (uint64_t)grid->nx * grid->ny * grid->nz;
    if (n == 0) return export_error("Invalid pressure grid dimensions");
    const uint64_t bytes = n * 16 * sizeof(float);
    const fs::path dir(directory);
    std::error_code ec;
    if (dir.has_parent_path() && !dir.parent_path().empty()) {
        fs::create_directories(dir.parent_path(), ec);
        if (ec) return export_error(ec.message());
    }
    // Exclusive creation protects previous exports and concurrent writers.
    if (mkdir(directory, 0777) != 0)
        return export_error(std::string("Create new frame directory ") + directory + ": " + std::strerror(errno));
    auto undo = [&](const std::string& msg) {
        std::error_code ignore;
        fs::remove_all(dir, ignore);
        return export_error(msg);
    };
    std::vector<float> host(n * 16);
    cudaError_t e = cudaMemcpy(host.data(), cells, bytes, cudaMemcpyDeviceToHost);
    if (e != cudaSuccess) return undo(std::string("field readback: ") + cudaGetErrorString(e));
    {
        FILE* f = fopen((dir / "fluid.bin").c_str(), "wb");
        if (!f) return undo(std::strerror(errno));
        const size_t wrote = fwrite(host.data(), 1, bytes, f);
        const bool ok = wrote == bytes && fclose(f) == 0;
        if (!ok) return undo("fluid.bin: short write");
    }
    const uint16_t probe = 1;
    const bool little = *reinterpret_cast<const uint8_t*>(&probe) == 1;
    const float o[3] = {origin_m ? origin_m[0] : 0.f, origin_m ? origin_m[1] : 0.f, origin_m ? origin_m[2] : 0.f};
    std::string m = "{\n";
    m += "  \"format_version\": 1,\n";
    m += "  \"step\": " + std::to_string(step) + ",\n";
    m += "  \"time_s\": " + json_number(time_s) + ",\n";
    m += "  \"origin_m\": [" + json_number(o[0]) + ", " + json_number(o[1]) + ", " + json_number(o[2]) + "],\n";
    m += "  \"cell_m\": " + json_number(grid->h) + ",\n";
    m += "  \"dims\": [" + std::to_string(grid->nx) + ", " + std::to_string(grid->ny) + ", " +
         std::to_string(grid->nz) + "],\n";
    m += std::string("  \"byte_order\": \"") + (little ? "little" : "big") + "\",\n";
    m += "  \"cell_order\": \"x fastest, then y, then z\",\n";
    m += "  \"files\": [{\"physics\": \"fluid\", \"file\": \"fluid.bin\", \"bytes\": " + std::to_string(bytes) +
         ", \"f32_components_per_cell\": 16}],\n";
    m += std::string("  \"moving_interface\": ") + (moving_interface ? "true" : "false") + ",\n";
    std::string kind = forcing_kind && forcing_kind[0] ? forcing_kind : "none";
    for (char c : kind)
        if (c == '"' || c == '\\' || (unsigned char)c < 0x20) return undo("forcing_kind must be a plain name");
    m += "  \"forcing_kind\": \"" + kind + "\"\n}\n";
    const fs::path staged = dir / "metadata.writing";
    {
        FILE* f = fopen(staged.c_str(), "wb");
        if (!f) return undo(std::strerror(errno));
        const bool ok = fwrite(m.data(), 1, m.size(), f) == m.size() && fclose(f) == 0;
        if (!ok) return undo("metadata: short write");
    }
    fs::rename(staged, dir / "metadata.json", ec);
    if (ec) return undo(ec.message());
    return 0;
}
