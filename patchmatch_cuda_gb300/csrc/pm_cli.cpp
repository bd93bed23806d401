// pm_cli.cpp -- command-line driver with the reference's surface (main.cpp:10-128):
//   pm_cli <config.ini>
// reads the [params] keys of main.cpp:47-85 (no Boost), the Middlebury image list
// (image.cpp:64-93: count, then per image "<file> K(9) R(9) t(3)"), PGM/PPM images (no
// OpenCV; colour is converted with BT.601 luma weights like cvtColor BGR2GRAY), runs the
// engine and writes outputFileName in the reference's depth format. blockDim_x/y are fixed
// by the engine. An NVM_V3 file (image.cpp:130-245) is read first, as the reference's main
// does: cameras from focal length, quaternion and centre (principal point at the image
// centre), and the reference image's depth range from the projected 3D points, widened by 25 %
// (the reference computes those ranges into a by-value copy and loses them; here they reach
// the engine).
#include <algorithm>
#include <cctype>
#include <cmath>
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

// Image::readNVM (image.cpp:130-245) with its depth ranges returned. Quaternion (w, x, y, z)
// to rotation as image.cpp:95-118; T = -R C (image.cpp:122-128); K = [f 0 W/2; 0 f H/2; 0 0 1].
bool read_nvm(const std::string &list, std::vector<Image> &imgs, std::vector<pm_view> &views,
              std::vector<std::pair<float, float>> &ranges)
{
    std::ifstream in(list);
    if (!in || in.peek() != 'N') return false;
    std::string header;
    in >> header;
    if (header.find("NVM_V3") == std::string::npos) return false;
    int ncam = 0;
    in >> ncam;
    if (!in || ncam <= 1) return false;
    imgs.assign((size_t)ncam, Image());
    views.assign((size_t)ncam, pm_view());
    std::vector<double> Rd((size_t)ncam * 9), Td((size_t)ncam * 3);
    for (int i = 0; i < ncam; ++i) {
        std::string name;
        double f, q[4], c[3], d[2];
        in >> name >> f >> q[0] >> q[1] >> q[2] >> q[3] >> c[0] >> c[1] >> c[2] >> d[0] >> d[1];
        if (!in) return false;
        const double qq = std::sqrt(q[0] * q[0] + q[1] * q[1] + q[2] * q[2] + q[3] * q[3]);
        double w = 1, x = 0, y = 0, z = 0;
        if (qq > 0) { w = q[0] / qq; x = q[1] / qq; y = q[2] / qq; z = q[3] / qq; }
        double *R = &Rd[(size_t)i * 9], *T = &Td[(size_t)i * 3];
        R[0] = w * w + x * x - z * z - y * y; R[1] = 2 * x * y - 2 * z * w; R[2] = 2 * y * w + 2 * z * x;
        R[3] = 2 * x * y + 2 * w * z; R[4] = y * y + w * w - z * z - x * x; R[5] = 2 * z * y - 2 * x * w;
        R[6] = 2 * x * z - 2 * y * w; R[7] = 2 * y * z + 2 * w * x; R[8] = z * z + w * w - y * y - x * x;
        for (int r = 0; r < 3; ++r) T[r] = -(R[3 * r] * c[0] + R[3 * r + 1] * c[1] + R[3 * r + 2] * c[2]);
        const std::string path = file_exists(name) ? name : dir_of(list) + "/" + name;
        if (!read_pnm(path, imgs[(size_t)i])) {
            std::printf("cannot read image %s (PGM/PPM, 8-bit)\n", path.c_str());
            return false;
        }
        pm_view &v = views[(size_t)i];
        v.gray = imgs[(size_t)i].px.data();
        v.width = v.stride = imgs[(size_t)i].w;
        v.height = imgs[(size_t)i].h;
        const float K[9] = {(float)f, 0.0f, (float)v.width / 2.0f, 0.0f, (float)f, (float)v.height / 2.0f,
                            0.0f, 0.0f, 1.0f};
        for (int k = 0; k < 9; ++k) { v.K[k] = K[k]; v.R[k] = (float)R[k]; }
        for (int k = 0; k < 3; ++k) v.t[k] = (float)T[k];
    }
    ranges.assign((size_t)ncam, std::make_pair(3.402823466e+38f, -3.402823466e+38f));
    int npoint = 0;
    in >> npoint;
    if (!in || npoint <= 0) return false;
    for (int i = 0; i < npoint; ++i) {
        float pt[3];
        int col[3], npj;
        in >> pt[0] >> pt[1] >> pt[2] >> col[0] >> col[1] >> col[2] >> npj;
        if (!in) return false;
        for (int j = 0; j < npj; ++j) {
            int cidx, fidx;
            float imx, imy;
            in >> cidx >> fidx >> imx >> imy;
            if (!in || cidx < 0 || cidx >= ncam) return false;
            // depth = third row of K [R | T] applied to the point (K's third row is 0 0 1)
            const pm_view &v = views[(size_t)cidx];
            const float depth = (float)((double)v.R[6] * pt[0] + (double)v.R[7] * pt[1] +
                                        (double)v.R[8] * pt[2] + (double)v.t[2]);
            if (depth <= 0) continue;  // image.cpp:211-212
            ranges[(size_t)cidx].first = std::min(ranges[(size_t)cidx].first, depth);
            ranges[(size_t)cidx].second = std::max(ranges[(size_t)cidx].second, depth);
        }
    }
    for (auto &r : ranges) {  // widen (image.cpp:222-235)
        if (r.first > r.second) continue;  // camera without projections
        const float size = r.second - r.first;
        float ratio = 0.25f, near_ = r.first - ratio * size;
        while (near_ <= 0) {
            ratio /= 1.1f;
            near_ = r.first - ratio * size;
        }
        r.first = near_;
        r.second += 0.25f * size;
    }
    return true;
}

bool read_middlebury(const std::string &list, std::vector<Image> &imgs, std::vector<pm_view> &views)
{
    std::ifstream in(list);
    if (!in) return false;
    int n = 0;
    in >> n;
    if (n < 1) return false;
    imgs.assign((size_t)n, Image());
    views.assign((size_t)n, pm_view());
    for (int i = 0; i < n; ++i) {
        std::string name;
        pm_view &v = views[(size_t)i];
        in >> name;
        for (float &k : v.K) in >> k;
        for (float &r : v.R) in >> r;
        for (float &t : v.t) in >> t;
        if (!in) return false;
        std::string path = file_exists(name) ? name : dir_of(list) + "/" + name;
        if (!read_pnm(path, imgs[(size_t)i])) {
            std::printf("cannot read image %s (PGM/PPM, 8-bit)\n", path.c_str());
            return false;
        }
        v.gray = imgs[(size_t)i].px.data();
        v.width = v.stride = imgs[(size_t)i].w;
        v.height = imgs[(size_t)i].h;
    }
    return true;
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
    // the engine's own keys (no counterpart in the reference's INI): slanted planes per pixel
    if (has("planes")) p.planes = std::atoi(get("planes").c_str());
    if (has("planeDepthStep")) p.plane_depth_step = std::strtof(get("planeDepthStep").c_str(), nullptr);
    if (has("planeSlopeStep")) p.plane_slope_step = std::strtof(get("planeSlopeStep").c_str(), nullptr);
    const std::string out = get("outputFileName");

    const std::string list = get("imageInfoFileName");
    std::vector<Image> imgs;
    std::vector<pm_view> views;
    std::vector<std::pair<float, float>> ranges;
    if (read_nvm(list, imgs, views, ranges)) {
        if (ref_id < 0 || ref_id >= (int)ranges.size() || ranges[(size_t)ref_id].first > ranges[(size_t)ref_id].second) {
            std::printf("NVM file has no 3D point seen by image %d\n", ref_id);
            return 1;
        }
        // main.cpp:117-121: the NVM range of the reference image replaces the configured one
        p.depth_near = ranges[(size_t)ref_id].first;
        p.depth_far = ranges[(size_t)ref_id].second;
        std::printf("using NVM files: depth range [%.9g, %.9g] for image %d\n", p.depth_near, p.depth_far, ref_id);
    } else if (read_middlebury(list, imgs, views)) {
        std::printf("using Middlebury files\n");
    } else {
        std::printf("cannot parse image files\n");
        return 1;
    }
    const int n = (int)views.size();

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
