// pm_cli.cpp -- command-line driver with the reference's surface (main.cpp:10-128):
//   pm_cli <config.ini>
// reads the [params] keys of main.cpp:47-85 (no Boost), the Middlebury image list
// (image.cpp:64-93: count, then per image "<file> K(9) R(9) t(3)"), PGM/PPM images (no
// OpenCV; colour is converted with BT.601 luma weights like cvtColor BGR2GRAY), runs the
// engine and writes outputFileName in the reference's depth format. blockDim_x/y are fixed
// by the engine. NVM input is not supported (the reference's NVM path discards its depth
// ranges, image.cpp:130 takes them by value).
#include <cctype>
#include <cstdio>
#include <cstdlib>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <vector>

#include "patchmatch_gb300.h"

namespace {

std::string trim(const std::string &s)
{
    size_t a = 0, b = s.size();
    while (a < b && std::isspace((unsigned char)s[a])) ++a;
    while (b > a && std::isspace((unsigned char)s[b - 1])) --b;
    return s.substr(a, b - a);
}

bool read_ini(const std::string &path, std::map<std::string, std::string> &kv)
{
    std::ifstream in(path);
    if (!in) return false;
    std::string line, section;
    while (std::getline(in, line)) {
        line = trim(line);
        if (line.empty() || line[0] == ';' || line[0] == '#') continue;
        if (line[0] == '[') {
            size_t e = line.find(']');
            if (e == std::string::npos) return false;
            section = trim(line.substr(1, e - 1));
            continue;
        }
        size_t eq = line.find('=');
        if (eq == std::string::npos) return false;
        kv[section + "." + trim(line.substr(0, eq))] = trim(line.substr(eq + 1));
    }
    return true;
}

struct Image {
    int w = 0, h = 0;
    std::vector<uint8_t> px;
};

bool read_token(std::istream &in, std::string &tok)
{
    tok.clear();
    int c;
    while ((c = in.get()) != EOF) {
        if (c == '#') {
            while ((c = in.get()) != EOF && c != '\n') {}
            continue;
        }
        if (!std::isspace(c)) { tok.push_back((char)c); break; }
    }
    while ((c = in.peek()) != EOF && !std::isspace(c)) tok.push_back((char)in.get());
    return !tok.empty();
}

bool read_pnm(const std::string &path, Image &img)
{
    std::ifstream in(path, std::ios::binary);
    if (!in) return false;
    std::string magic, sw, sh, smax;
    if (!read_token(in, magic) || !read_token(in, sw) || !read_token(in, sh) || !read_token(in, smax)) return false;
    if ((magic != "P5" && magic != "P6") || std::atoi(smax.c_str()) != 255) return false;
    in.get();
    img.w = std::atoi(sw.c_str());
    img.h = std::atoi(sh.c_str());
    if (img.w <= 0 || img.h <= 0) return false;
    const size_t n = (size_t)img.w * img.h;
    img.px.resize(n);
    if (magic == "P5") {
        in.read((char *)img.px.data(), (std::streamsize)n);
        return (size_t)in.gcount() == n;
    }
    std::vector<uint8_t> rgb(3 * n);
    in.read((char *)rgb.data(), (std::streamsize)rgb.size());
    if ((size_t)in.gcount() != rgb.size()) return false;
    for (size_t i = 0; i < n; ++i) {
        const unsigned r = rgb[3 * i], g = rgb[3 * i + 1], b = rgb[3 * i + 2];
        img.px[i] = (uint8_t)((r * 4899u + g * 9617u + b * 1868u + 8192u) >> 14);
    }
    return true;
}

std::string dir_of(const std::string &p)
{
    size_t s = p.find_last_of('/');
    return s == std::string::npos ? std::string(".") : p.substr(0, s);
}

bool file_exists(const std::string &p)
{
    std::ifstream f(p);
    return (bool)f;
}

}  // namespace

int main(int argc, char **argv)
{
    if (argc < 2) {
        std::printf("Initialization file is mandatory to run the code\n");
        return 1;
    }
    std::map<std::string, std::string> kv;
    if (!read_ini(argv[1], kv)) {
        std::printf("Problems with config file: cannot parse %s\n", argv[1]);
        return 1;
    }
    const char *required[] = {"imageInfoFileName", "refImageId", "halfWindowSize", "numOfSamples",
                              "SPMAlpha", "gaussianSigma", "numOfIterations", "outputFileName"};
    for (const char *k : required)
        if (!kv.count(std::string("params.") + k)) {
            std::printf("Problems with config file: No such node (params.%s)\n", k);
            return 1;
        }
    auto get = [&](const char *k) { return kv[std::string("params.") + k]; };
    auto has = [&](const char *k) { return kv.count(std::string("params.") + k) > 0; };

    pm_params p;
    pm_default_params(&p);
    p.depth_near = has("depthRangeNear") ? std::strtof(get("depthRangeNear").c_str(), nullptr) : -1.0f;
    p.depth_far = has("depthRangeFar") ? std::strtof(get("depthRangeFar").c_str(), nullptr) : -1.0f;
    p.gpu_id = has("gpuId") ? std::atoi(get("gpuId").c_str()) : -1;
    if (has("orientationX") && has("orientationZ")) {
        p.orientation_x = std::strtof(get("orientationX").c_str(), nullptr);
        p.orientation_z = std::strtof(get("orientationZ").c_str(), nullptr);
    }
    const int ref_id = std::atoi(get("refImageId").c_str());
    p.half_window = std::atoi(get("halfWindowSize").c_str());
    p.num_samples = std::atoi(get("numOfSamples").c_str());
    p.sp_alpha = std::strtof(get("SPMAlpha").c_str(), nullptr);
    p.gaussian_sigma = std::strtof(get("gaussianSigma").c_str(), nullptr);
    p.num_iterations = std::atoi(get("numOfIterations").c_str());
    if (has("prefilter")) p.prefilter = std::atoi(get("prefilter").c_str());
    if (has("seed")) p.seed = std::strtoull(get("seed").c_str(), nullptr, 10);
    if (has("precision")) p.precision = std::atoi(get("precision").c_str());
    const std::string out = get("outputFileName");

    const std::string list = get("imageInfoFileName");
    std::ifstream in(list);
    if (!in) {
        std::printf("cannot parse image files\n");
        return 1;
    }
    int n = 0;
    in >> n;
    if (n < 1) {
        std::printf("cannot parse image files\n");
        return 1;
    }
    std::vector<Image> imgs((size_t)n);
    std::vector<pm_view> views((size_t)n);
    for (int i = 0; i < n; ++i) {
        std::string name;
        pm_view &v = views[(size_t)i];
        in >> name;
        for (float &k : v.K) in >> k;
        for (float &r : v.R) in >> r;
        for (float &t : v.t) in >> t;
        if (!in) {
            std::printf("cannot parse image files\n");
            return 1;
        }
        std::string path = file_exists(name) ? name : dir_of(list) + "/" + name;
        if (!read_pnm(path, imgs[(size_t)i])) {
            std::printf("cannot read image %s (PGM/PPM, 8-bit)\n", path.c_str());
            return 1;
        }
        v.gray = imgs[(size_t)i].px.data();
        v.width = v.stride = imgs[(size_t)i].w;
        v.height = imgs[(size_t)i].h;
    }
    std::printf("using Middlebury files\n");

    pm_handle *h = nullptr;
    pm_status s = pm_create(views.data(), n, ref_id, &p, &h);
    if (s != PM_OK) {
        std::printf("Error: %s %s\n", pm_status_string(s), h ? pm_last_error(h) : "");
        return 1;
    }
    s = pm_run(h);
    if (s == PM_OK) s = pm_save_depth(h, out.c_str());
    if (s != PM_OK) {
        std::printf("Error: %s: %s\n", pm_status_string(s), pm_last_error(h));
        pm_destroy(h);
        return 1;
    }
    pm_stats st;
    pm_get_stats(h, &st);
    std::printf("depth map %s: %.3f ms, %llu cost evaluations\n", out.c_str(), st.ms_total,
                st.cost_evals);
    pm_destroy(h);
    return 0;
}
