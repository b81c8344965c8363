// main.cpp — the `pt` command-line program on top of libptgpu.so.
//
// Keeps the reference's interface (src/main.cpp:16-128, src/argparse.cpp):
//   pt [--headless] [-w W] [-h H] [-s SPP] [-b BOUNCES] [-o OUT] [-f png|hdr] [-t T] scene.scn
// with the same defaults (s=32, b=2, w=h=400, f=png), the same error
// messages and exit codes, and the same stdout lines (scene.cpp:505-516,
// ptdispatch.cpp:67-75).  Only headless rendering exists here; the
// interactive viewer of the reference needs a window system.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <iostream>
#include <optional>
#include <regex>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../../include/pt_gpu.h"
#include "../../../include/pt_scene.h"

namespace {

enum class Kind { STRING, SWITCH, INTEGER, DECIMAL };

struct Option {
    std::string name, short_name;
    Kind kind;
    std::string description;
    std::optional<std::string> value;
};

struct Parser {
    std::vector<Option> options;
    std::unordered_map<std::string, size_t> by_name, by_short;

    void add(const std::string& n, const std::string& s, Kind k, const std::string& d)
    {
        by_name[n] = options.size();
        if (!s.empty())
            by_short[s] = options.size();
        options.push_back({n, s, k, d, std::nullopt});
    }
    // argparse.cpp:61-101: --long [value], -x value or -xVALUE, "--" ends options.
    void parse(int argc, char** argv, std::vector<std::string>& rest)
    {
        bool ended = false;
        for (int i = 1; i < argc; i++) {
            std::string t = argv[i];
            if (!ended && t.size() >= 3 && t[0] == '-' && t[1] == '-') {
                if (!by_name.count(t))
                    throw std::runtime_error("Unknown option " + t + ".");
                Option& o = options[by_name[t]];
                if (o.kind == Kind::SWITCH) {
                    o.value = "true";
                } else {
                    if (++i >= argc)
                        throw std::runtime_error("Option " + t + " has no value.");
                    o.value = argv[i];
                }
            } else if (!ended && t.size() >= 2 && t[0] == '-' && t[1] != '-') {
                std::string k = t.substr(0, 2);
                if (!by_short.count(k))
                    throw std::runtime_error("Unknown option " + k + ".");
                Option& o = options[by_short[k]];
                if (o.kind == Kind::SWITCH) {
                    if (t.size() != 2)
                        throw std::runtime_error("Switch option " + k + " has a value.");
                    o.value = "true";
                } else if (t.size() == 2) {
                    if (++i >= argc)
                        throw std::runtime_error("Option " + t + " has no value.");
                    o.value = argv[i];
                } else {
                    o.value = t.substr(2);
                }
            } else if (t == "--") {
                ended = true;
            } else {
                rest.push_back(t);
            }
        }
    }
    const Option& get(const std::string& n) const { return options.at(by_name.at(n)); }
    std::optional<int> integer(const std::string& n) const
    {
        const Option& o = get(n);
        if (!o.value)
            return std::nullopt;
        if (!std::regex_match(*o.value, std::regex("[\\-\\+]?[0-9]+")))
            throw std::runtime_error("The value of option " + n + " was not an integer: " + *o.value);
        return std::stoi(*o.value);
    }
    std::optional<float> decimal(const std::string& n) const
    {
        const Option& o = get(n);
        if (!o.value)
            return std::nullopt;
        if (!std::regex_match(*o.value, std::regex("[\\-\\+]?[0-9]+(\\.[0-9]*)?")))
            throw std::runtime_error("The value of option " + n + " was not a decimal number: " + *o.value);
        return std::stof(*o.value);
    }
    bool flag(const std::string& n) const { return get(n).value == std::string("true"); }
    std::optional<std::string> str(const std::string& n) const { return get(n).value; }
    std::string help() const
    {
        std::string r = "Options:";
        for (const Option& o : options) {
            r += "\n  " + o.name;
            if (!o.short_name.empty())
                r += ", " + o.short_name;
            r += "\t" + o.description;
        }
        return r;
    }
};

void print_help(const std::string& program, const Parser& p)
{
    std::cout << "Usage: " << program << " [options] path-to-scene\n" << p.help() << std::endl;
}

int check(int rc, pt_ctx* ctx, const char* what)
{
    if (rc != PT_OK) {
        std::cerr << "Error: " << what << ": " << pt_last_error(ctx) << std::endl;
        return 1;
    }
    return 0;
}

} // namespace

int main(int argc, char** argv)
{
    Parser parser;
    parser.add("--help", "", Kind::SWITCH, "Displays help.");
    parser.add("--width", "-w", Kind::INTEGER, "The width of the rendered image.");
    parser.add("--height", "-h", Kind::INTEGER, "The height of the rendered image.");
    parser.add("--headless", "", Kind::SWITCH, "Run without window and user interface.");
    parser.add("--samples", "-s", Kind::INTEGER, "Number of samples to take.");
    parser.add("--bounces", "-b", Kind::INTEGER, "Maximum number of ray bounces.");
    parser.add("--out", "-o", Kind::STRING, "Specifies in which file to place the output.");
    parser.add("--format", "-f", Kind::STRING, "The image format of the output file.");
    parser.add("--time", "-t", Kind::DECIMAL, "The maximum rendering time.");

    std::vector<std::string> args;
    int samples, bounces, width, height;
    std::optional<std::string> out;
    std::string format;
    try {
        parser.parse(argc, argv, args);
        if (parser.flag("--help")) {
            print_help(argv[0], parser);
            return 0;
        }
        if (args.empty()) {
            std::cerr << "Error: Expected path to scene." << std::endl;
            print_help(argv[0], parser);
            return 1;
        }
        if (args.size() > 1) {
            std::cerr << "Error: Unexpected number of arguments." << std::endl;
            print_help(argv[0], parser);
            return 1;
        }
        samples = parser.integer("--samples").value_or(32);
        if (samples < 1) {
            std::cerr << "Error: Invalid sample count: " << samples << "." << std::endl;
            return 1;
        }
        bounces = parser.integer("--bounces").value_or(2);
        if (bounces < 0) {
            std::cerr << "Error: Invalid number of ray bounces: " << bounces << "." << std::endl;
            return 1;
        }
        out = parser.str("--out");
        if (parser.flag("--headless") && !out) {
            std::cerr << "Error: No output file was given (required for headless execution)." << std::endl;
            return 1;
        }
        width = parser.integer("--width").value_or(400);
        height = parser.integer("--height").value_or(400);
        if (width < 1 || height < 1) {
            std::cerr << "Error: Invalid dimensions: (" << width << ", " << height << ")." << std::endl;
            return 1;
        }
        format = parser.str("--format").value_or("png");
        if (!(format == "png" || format == "PNG" || format == "hdr" || format == "HDR")) {
            std::cerr << "Error: Output format is invalid: " << format << std::endl;
            return 1;
        }
        (void)parser.decimal("--time"); // parsed but unused, as in the reference
    } catch (const std::exception& e) {
        std::cerr << "Error: " << e.what() << std::endl;
        print_help(argv[0], parser);
        return 1;
    }
    if (!parser.flag("--headless")) {
        std::cerr << "Error: the interactive viewer is not part of this build; use --headless." << std::endl;
        return 1;
    }

    pt_host_scene* scene = pt_scene_load(args[0].c_str());
    if (!scene) {
        std::cerr << "Error: " << pt_scene_last_error() << std::endl;
        return 1;
    }
    char details[1024];
    pt_scene_details(scene, details, sizeof(details));
    std::cout << details << std::endl;

    pt_ctx* ctx = pt_create(0);
    if (!ctx) {
        std::cerr << "Error: " << pt_last_error(nullptr) << std::endl;
        pt_scene_free(scene);
        return 1;
    }
    pt_scene_view view;
    int rc = pt_scene_pack(scene, &view);
    if (rc != PT_OK) {
        std::cerr << "Error: " << pt_scene_last_error() << std::endl;
        return 1;
    }
    if (check(pt_upload_scene(ctx, &view), ctx, "scene upload") || check(pt_build_accel(ctx, nullptr), ctx, "acceleration structure"))
        return 1;
    pt_camera_desc cam;
    pt_scene_camera(scene, &cam);
    pt_render_params params{};
    pt_camera_params(&cam, (uint32_t)width, (uint32_t)height, &params);
    params.sample_index = 0;
    params.samples = (uint32_t)samples;
    params.max_bounces = (uint32_t)bounces;
    params.accum_mode = PT_ACCUM_FP32;
    params.kernel = PT_KERNEL_AUTO;
    params.rr_start = 1;

    bool png = format == "png" || format == "PNG";
    std::vector<float> pixels((size_t)width * height * 4);
    auto start = std::chrono::high_resolution_clock::now();
    if (check(pt_render(ctx, &params, nullptr), ctx, "render"))
        return 1;
    if (png && check(pt_tonemap(ctx), ctx, "tone map"))
        return 1;
    if (check(pt_read_image(ctx, pixels.data(), (size_t)width * 16, 0), ctx, "read-back"))
        return 1;
    float taken = std::chrono::duration<float>(std::chrono::high_resolution_clock::now() - start).count();
    std::cout << "Rendering took " << taken << " seconds with " << samples << " samples taken per pixel.\n";
    std::cout << samples / taken << " samples per second.\n";
    std::cout << "Writing image to " << *out << std::endl;
    rc = png ? pt_write_png(out->c_str(), pixels.data(), (uint32_t)width, (uint32_t)height)
             : pt_write_hdr(out->c_str(), pixels.data(), (uint32_t)width, (uint32_t)height);
    pt_destroy(ctx);
    pt_scene_free(scene);
    if (rc != PT_OK) {
        std::cerr << "Error: Could not write " << (png ? "PNG" : "HDR") << " file." << std::endl;
        return 1;
    }
    return 0;
}
