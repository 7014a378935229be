// ffvship.cpp -- command-line scorer with the reference FFVship's interface
// (src/FFVship.cpp:202-519, src/ffvship_utility/ffmpegmain.hpp:782-873).
//
// Same flags, per-frame JSON format and statistics block as the reference. Decoding: the
// reference decodes any container with ffms2 and converts colour with zimg on the CPU; neither
// library is available here, so this tool reads YUV4MPEG2 (.y4m) files (4:2:0 / 4:2:2 / 4:4:4,
// 8-16 bit) and hands the planes to the GPU front-end (Vship_SSIMU2SetYuvFormat +
// Vship_ComputeSSIMU2Yuv, and the Butteraugli pair), which converts colour on the device.
//
// Pipeline (as the reference's): reader threads fill a bounded frame-pair queue, GPU worker
// threads (one handler each) score pairs, the main thread aggregates results in frame order.
#include "../../include/VshipAPI.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <thread>
#include <vector>

namespace {

const char* kVersion = "vship_gb300 ffvship 3.1.0";

// ------------------------------------------------------------------------------------------
// YUV4MPEG2 reader: C420jpeg / C420 (center siting), C420mpeg2 (left), C420paldv (top-left),
// C420pN / C422[pN] / C444[pN] (N = 9..16; chroma siting unspecified, read as left, the
// reference's default, ffmpegToZimgFormat.hpp:224-227), optional XCOLORRANGE=FULL. Y4M carries no
// matrix, so the reference's guess by height applies (matrix 2).
struct Y4M {
    std::string path;
    int w = 0, h = 0, bits = 8, ssw = 1, ssh = 1, loc = 0, full = 0;
    int64_t header_len = 0, frame_bytes = 0, nframes = 0;
    int64_t frame_stride = 0;  // "FRAME\n" + payload

    int64_t cw() const { return ssw ? (w + 1) / 2 : w; }
    int64_t ch() const { return ssh ? (h + 1) / 2 : h; }

    bool open(const std::string& p, std::string& err) {
        path = p;
        FILE* f = std::fopen(p.c_str(), "rb");
        if (!f) {
            err = "cannot open " + p;
            return false;
        }
        std::string line;
        int c;
        while ((c = std::fgetc(f)) != EOF && c != '\n') line.push_back((char)c);
        if (line.rfind("YUV4MPEG2", 0) != 0) {
            std::fclose(f);
            err = p + " is not a YUV4MPEG2 file";
            return false;
        }
        header_len = (int64_t)line.size() + 1;
        std::istringstream ss(line);
        std::string tok;
        std::string cs = "420jpeg";
        while (ss >> tok) {
            if (tok[0] == 'W') w = std::atoi(tok.c_str() + 1);
            else if (tok[0] == 'H') h = std::atoi(tok.c_str() + 1);
            else if (tok[0] == 'C') cs = tok.substr(1);
            else if (tok == "XCOLORRANGE=FULL") full = 1;
        }
        const std::string sub = cs.substr(0, 3);
        if (sub == "420") {
            ssw = ssh = 1;
        } else if (sub == "422") {
            ssw = 1;
            ssh = 0;
        } else if (sub == "444") {
            ssw = ssh = 0;
        } else {
            std::fclose(f);
            err = p + ": unsupported YUV4MPEG2 colorspace C" + cs;
            return false;
        }
        const std::string rest = cs.substr(3);
        bits = 8;
        loc = 0;
        if (rest.empty() || rest == "jpeg") {
            loc = ssw ? 1 : 0;  // 4:2:0 JPEG / MPEG-1 siting: center
        } else if (rest == "mpeg2") {
            loc = 0;
        } else if (rest == "paldv") {
            loc = 2;
        } else if (rest[0] == 'p') {
            bits = std::atoi(rest.c_str() + 1);
        } else {
            std::fclose(f);
            err = p + ": unsupported YUV4MPEG2 colorspace C" + cs;
            return false;
        }
        if (bits < 8 || bits > 16 || w <= 0 || h <= 0) {
            std::fclose(f);
            err = p + ": bad bit depth or missing W/H";
            return false;
        }
        frame_bytes = ((int64_t)w * h + 2 * cw() * ch()) * (bits > 8 ? 2 : 1);
        // frame header: "FRAME" plus optional parameters up to '\n'
        std::fseek(f, header_len, SEEK_SET);
        std::string fh;
        while ((c = std::fgetc(f)) != EOF && c != '\n') fh.push_back((char)c);
        if (fh.rfind("FRAME", 0) != 0) {
            std::fclose(f);
            err = p + ": no FRAME marker";
            return false;
        }
        frame_stride = (int64_t)fh.size() + 1 + frame_bytes;
        std::fseek(f, 0, SEEK_END);
        const int64_t size = std::ftell(f);
        std::fclose(f);
        nframes = (size - header_len) / frame_stride;
        return true;
    }

    // Reads frame k. Samples stay as stored (bytes for 8 bits, 16-bit containers above), except
    // that `to_bits` > bits widens limited-range samples to that depth by a shift, which keeps
    // every decoded value exactly (both map code 16 << (d - 8) to 0 and 235 << (d - 8) to 1).
    bool read(int64_t k, std::vector<uint8_t>& out, int to_bits, std::string& err) const {
        FILE* f = std::fopen(path.c_str(), "rb");
        if (!f) {
            err = "cannot open " + path;
            return false;
        }
        const int64_t off = header_len + k * frame_stride + (frame_stride - frame_bytes);
        std::fseek(f, off, SEEK_SET);
        const int64_t n = frame_bytes / (bits > 8 ? 2 : 1);
        bool ok;
        if (to_bits == bits) {
            out.resize(frame_bytes);
            ok = std::fread(out.data(), 1, frame_bytes, f) == (size_t)frame_bytes;
        } else {
            std::vector<uint8_t> raw(frame_bytes);
            ok = std::fread(raw.data(), 1, frame_bytes, f) == (size_t)frame_bytes;
            out.resize(n * 2);
            uint16_t* o16 = reinterpret_cast<uint16_t*>(out.data());
            const int sh = to_bits - bits;
            for (int64_t i = 0; i < n; i++) {
                const unsigned v = bits > 8 ? (unsigned)raw[2 * i] | ((unsigned)raw[2 * i + 1] << 8) : raw[i];
                o16[i] = (uint16_t)(v << sh);
            }
        }
        std::fclose(f);
        if (!ok) err = path + ": short read at frame " + std::to_string(k);
        return ok;
    }
};

struct Crop {
    int top = 0, bottom = 0, left = 0, right = 0;
};

// planes of a (cropped) frame inside a read buffer of `bytes` per sample
struct PlaneView {
    const uint8_t* p[3];
    int64_t stride[3];
};
PlaneView view(const std::vector<uint8_t>& buf, const Y4M& y, int bytes, const Crop& c) {
    const int64_t w = y.w, h = y.h, cw = y.cw(), ch = y.ch();
    const uint8_t* Y = buf.data();
    const uint8_t* U = Y + (size_t)w * h * bytes;
    const uint8_t* V = U + (size_t)cw * ch * bytes;
    const int cl = y.ssw ? c.left / 2 : c.left, ct = y.ssh ? c.top / 2 : c.top;
    PlaneView v;
    v.p[0] = Y + ((size_t)c.top * w + c.left) * bytes;
    v.p[1] = U + ((size_t)ct * cw + cl) * bytes;
    v.p[2] = V + ((size_t)ct * cw + cl) * bytes;
    v.stride[0] = w * bytes;
    v.stride[1] = v.stride[2] = cw * bytes;
    return v;
}

// ------------------------------------------------------------------------------------------
// options (ffmpegmain.hpp:796-830)
enum class Metric { SSIMU2, Butteraugli };

struct Options {
    std::string source, encoded, json, metric_name = "SSIMULACRA2";
    bool live = false, list_gpu = false, version = false;
    int start = 0, end = -1, every = 1, encoded_offset = 0;
    std::string source_indices, encoded_indices;
    Crop crop_src, crop_enc;
    float intensity = 203.f;
    int qnorm = 2, threads = 2, gpu_threads = 3, gpu_id = 0;
    Metric metric = Metric::SSIMU2;
};

std::vector<std::string> read_config_file(const std::string& path) {
    std::ifstream f(path);
    std::string line;
    std::getline(f, line);
    std::istringstream ss(line);
    std::vector<std::string> out;
    std::string tok;
    while (ss >> tok) out.push_back(tok);
    return out;
}

void usage() {
    std::cerr << "usage: ffvship -s SOURCE.y4m -e ENCODED.y4m [-m SSIMULACRA2|Butteraugli] [--json FILE]\n"
                 "  [--live-score-output] [--start N] [--end N] [--every N] [--encoded-offset N]\n"
                 "  [--source-indices a,b,..] [--encoded-indices a,b,..] [--crop{Top,Bottom,Left,Right}{Source,Encoded} N]\n"
                 "  [--intensity-target NITS] [--qnorm Q] [-t READERS] [-g GPU_THREADS] [--gpu-id N]\n"
                 "  [--list-gpu] [--version] [--config-file FILE]\n";
}

bool parse_ints(const std::string& s, std::vector<int>& out) {
    out.clear();
    if (s.empty()) return true;
    std::stringstream ss(s);
    std::string tok;
    while (std::getline(ss, tok, ',')) {
        char* end = nullptr;
        long v = std::strtol(tok.c_str(), &end, 10);
        if (!end || *end) return false;
        out.push_back((int)v);
    }
    return true;
}

int parse(int argc, char** argv, Options& o) {
    std::vector<std::string> a(argv + 1, argv + argc);
    for (size_t i = 0; i < a.size(); i++)
        if (a[i] == "--config-file" && i + 1 < a.size()) {
            std::vector<std::string> extra = read_config_file(a[i + 1]);
            a.erase(a.begin() + i, a.begin() + i + 2);
            a.insert(a.end(), extra.begin(), extra.end());
            break;
        }
    auto need = [&](size_t& i) -> const std::string& {
        if (i + 1 >= a.size()) throw std::runtime_error("missing value for " + a[i]);
        return a[++i];
    };
    std::map<std::string, int*> ints = {
        {"--start", &o.start}, {"--end", &o.end}, {"--every", &o.every}, {"--encoded-offset", &o.encoded_offset},
        {"--qnorm", &o.qnorm}, {"--threads", &o.threads}, {"-t", &o.threads}, {"--gpu-threads", &o.gpu_threads},
        {"-g", &o.gpu_threads}, {"--gpu-id", &o.gpu_id},
        {"--cropTopSource", &o.crop_src.top}, {"--cropBottomSource", &o.crop_src.bottom},
        {"--cropLeftSource", &o.crop_src.left}, {"--cropRightSource", &o.crop_src.right},
        {"--cropTopEncoded", &o.crop_enc.top}, {"--cropBottomEncoded", &o.crop_enc.bottom},
        {"--cropLeftEncoded", &o.crop_enc.left}, {"--cropRightEncoded", &o.crop_enc.right}};
    try {
        for (size_t i = 0; i < a.size(); i++) {
            const std::string& k = a[i];
            if (k == "--source" || k == "-s") o.source = need(i);
            else if (k == "--encoded" || k == "-e") o.encoded = need(i);
            else if (k == "--metric" || k == "-m") o.metric_name = need(i);
            else if (k == "--json") o.json = need(i);
            else if (k == "--live-score-output") o.live = true;
            else if (k == "--list-gpu") o.list_gpu = true;
            else if (k == "--version") o.version = true;
            else if (k == "--source-indices") o.source_indices = need(i);
            else if (k == "--encoded-indices") o.encoded_indices = need(i);
            else if (k == "--intensity-target") o.intensity = std::stof(need(i));
            else if (k == "--source-index" || k == "--encoded-index") need(i);  // ffms2 index files: unused
            else if (k == "--cache-index") {
            } else if (ints.count(k)) *ints[k] = std::stoi(need(i));
            else {
                std::cerr << "Unknown argument " << k << "\n";
                usage();
                return 1;
            }
        }
    } catch (const std::exception& e) {
        std::cerr << e.what() << "\n";
        return 1;
    }
    std::string m = o.metric_name;
    std::transform(m.begin(), m.end(), m.begin(), ::tolower);
    if (m == "ssimulacra2" || m == "ssimu2") o.metric = Metric::SSIMU2;
    else if (m == "butteraugli") o.metric = Metric::Butteraugli;
    else {
        std::cerr << "Unknown metric type. Expected 'SSIMULACRA2' or 'Butteraugli'.\n";
        return 1;
    }
    return 0;
}

// FFVship.cpp:142-200
void print_stats(const std::vector<float>& data, const std::string& label) {
    if (data.empty()) return;
    std::vector<float> s = data;
    std::sort(s.begin(), s.end());
    const size_t n = s.size();
    double avg = 0, sq = 0;
    for (float v : s) avg += v;
    avg /= n;
    for (float v : s) sq += (v - avg) * (v - avg);
    const double sd = std::sqrt(sq / n);
    std::vector<std::pair<std::string, double>> st = {{"Average", avg},          {"Standard Deviation", sd},
                                                      {"Median", s[n / 2]},      {"5th percentile", s[n / 20]},
                                                      {"95th percentile", s[19 * n / 20]}, {"Minimum", s.front()},
                                                      {"Maximum", s.back()}};
    size_t lw = 0;
    for (auto& kv : st) lw = std::max(lw, kv.first.size());
    const int vw = 12, total = (int)lw + 3 + vw;
    const int pad = std::max(0, (total - (int)label.size()) / 2);
    std::cout << std::string(pad, '-') << label << std::string(std::max(0, total - pad - (int)label.size()), '-')
              << "\n";
    for (auto& kv : st)
        std::cout << std::setw((int)lw) << std::right << kv.first << " : " << std::setw(vw) << std::right
                  << std::fixed << std::setprecision(6) << kv.second << "\n";
    std::cout << "\n";
}

struct Job {
    int idx;
    int64_t src_frame, enc_frame;
};

template <typename T>
class Queue {
    std::mutex mu;
    std::condition_variable cv;
    std::vector<T> items;
    bool closed = false;
    size_t cap;

public:
    explicit Queue(size_t c) : cap(c) {}
    void push(T v) {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return items.size() < cap || closed; });
        items.push_back(std::move(v));
        cv.notify_all();
    }
    bool pop(T& out) {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return !items.empty() || closed; });
        if (items.empty()) return false;
        out = std::move(items.front());
        items.erase(items.begin());
        cv.notify_all();
        return true;
    }
    void close() {
        std::lock_guard<std::mutex> lk(mu);
        closed = true;
        cv.notify_all();
    }
};

struct Loaded {
    int idx;
    std::vector<uint8_t> src, enc;
};

std::string err_text(Vship_Exception e) {
    int n = Vship_GetErrorMessage(e, nullptr, 0);
    std::string s(n, '\0');
    Vship_GetErrorMessage(e, &s[0], n);
    s.resize(n - 1);
    return s;
}

}  // namespace

int main(int argc, char** argv) {
    Options o;
    if (parse(argc, argv, o)) return 1;
    if (o.version) {
        std::cout << kVersion << "\n";
        return 0;
    }
    if (o.list_gpu) {
        int n = 0;
        Vship_Exception e = Vship_GetDeviceCount(&n);
        if (e != Vship_NoError) {
            std::cerr << err_text(e) << "\n";
            return 1;
        }
        for (int i = 0; i < n; i++) {
            Vship_DeviceInfo info;
            if (Vship_GetDeviceInfo(&info, i) == Vship_NoError) std::cout << "GPU " << i << ": " << info.name << "\n";
        }
        return 0;
    }
    if (o.source.empty() || o.encoded.empty()) {
        std::cerr << (o.source.empty() ? "Source file is not specified\n" : "Encoded file is not specified\n");
        usage();
        return 1;
    }
    Y4M src, enc;
    std::string err;
    if (!src.open(o.source, err) || !enc.open(o.encoded, err)) {
        std::cerr << err << "\n";
        return 1;
    }
    const Crop& cs = o.crop_src;
    const Crop& ce = o.crop_enc;
    for (const Crop* c : {&cs, &ce})
        if ((((c->top | c->bottom) & 1) && src.ssh) || (((c->left | c->right) & 1) && src.ssw)) {
            std::cerr << "crops must be even along subsampled chroma directions\n";
            return 1;
        }
    // one Y'CbCr format for both files: equal formats, or limited-range ones that differ only in
    // depth (the shallower one is widened, exactly)
    if (src.ssw != enc.ssw || src.ssh != enc.ssh || src.loc != enc.loc || src.full != enc.full ||
        (src.bits != enc.bits && src.full)) {
        std::cerr << "DifferingInputType: source and encoded Y'CbCr formats differ\n";
        return 1;
    }
    const int bits = std::max(src.bits, enc.bits);
    const int bytes = bits > 8 ? 2 : 1;
    Vship_YuvFormat yfmt{bits, src.ssw, src.ssh, 2, src.full, src.loc, 2, 2};
    const int w = src.w - cs.left - cs.right, h = src.h - cs.top - cs.bottom;
    if (w != enc.w - ce.left - ce.right || h != enc.h - ce.top - ce.bottom || w <= 0 || h <= 0) {
        std::cerr << "DifferingInputType: source and encoded differ in size after cropping\n";
        return 1;
    }
    // frame selection (start / end / every / offset / explicit index lists)
    std::vector<int> sidx, eidx;
    if (!parse_ints(o.source_indices, sidx) || !parse_ints(o.encoded_indices, eidx)) {
        std::cerr << "Invalid integer found in --source-indices / --encoded-indices\n";
        return 1;
    }
    const int end = o.end < 0 ? (int)src.nframes : std::min<int>(o.end, (int)src.nframes);
    std::vector<Job> jobs;
    if (sidx.empty())
        for (int i = o.start; i < end; i += std::max(1, o.every)) sidx.push_back(i);
    if (eidx.empty()) eidx = sidx;
    if (eidx.size() != sidx.size()) {
        std::cerr << "--source-indices and --encoded-indices differ in length\n";
        return 1;
    }
    for (size_t k = 0; k < sidx.size(); k++) {
        const int64_t sf = sidx[k], ef = (int64_t)eidx[k] + o.encoded_offset;
        if (sf < 0 || sf >= src.nframes || ef < 0 || ef >= enc.nframes) continue;
        jobs.push_back({(int)jobs.size(), sf, ef});
    }
    const int nframes = (int)jobs.size();
    if (Vship_Exception e = Vship_SetDevice(o.gpu_id); e != Vship_NoError) {
        std::cerr << err_text(e) << "\n";
        return 1;
    }
    if (Vship_Exception e = Vship_GPUFullCheck(o.gpu_id); e != Vship_NoError) {
        std::cerr << err_text(e) << "\n";
        return 1;
    }
    const int nres = o.metric == Metric::Butteraugli ? 3 : 1;
    std::vector<float> scores((size_t)nframes * nres, 0.f);
    std::atomic<int> next_job{0}, done{0}, failed{0};
    Queue<Loaded> frames(std::max(2, 2 * o.gpu_threads));
    auto t0 = std::chrono::high_resolution_clock::now();
    std::vector<std::thread> readers;
    std::atomic<int> readers_left{std::max(1, o.threads)};
    for (int r = 0; r < std::max(1, o.threads); r++)
        readers.emplace_back([&] {
            for (;;) {
                const int k = next_job.fetch_add(1);
                if (k >= nframes) break;
                Loaded l;
                l.idx = k;
                std::string e;
                if (!src.read(jobs[k].src_frame, l.src, bits, e) || !enc.read(jobs[k].enc_frame, l.enc, bits, e)) {
                    std::cerr << e << "\n";
                    failed = 1;
                    continue;
                }
                frames.push(std::move(l));
            }
            if (--readers_left == 0) frames.close();
        });
    std::mutex out_mu;
    if (o.live) std::cout << nframes << "\n";
    std::vector<std::thread> workers;
    for (int g = 0; g < std::max(1, o.gpu_threads); g++)
        workers.emplace_back([&] {
            Vship_SetDevice(o.gpu_id);
            Vship_SSIMU2Handler hs{};
            Vship_ButteraugliHandler hb{};
            Vship_Exception e = o.metric == Metric::SSIMU2 ? Vship_SSIMU2Init(&hs, w, h)
                                                           : Vship_ButteraugliInitv2(&hb, w, h, o.qnorm, o.intensity);
            if (e == Vship_NoError)
                e = o.metric == Metric::SSIMU2 ? Vship_SSIMU2SetYuvFormat(hs, &yfmt)
                                               : Vship_ButteraugliSetYuvFormat(hb, &yfmt);
            if (e != Vship_NoError) {
                std::cerr << err_text(e) << "\n";
                failed = 1;
            }
            Loaded l;
            while (frames.pop(l)) {
                if (e != Vship_NoError) continue;
                PlaneView a = view(l.src, src, bytes, cs), b = view(l.enc, enc, bytes, ce);
                Vship_Exception rc;
                if (o.metric == Metric::SSIMU2) {
                    double s = 0;
                    rc = Vship_ComputeSSIMU2Yuv(hs, &s, a.p, a.stride, b.p, b.stride);
                    scores[l.idx] = (float)s;
                } else {
                    double n[3] = {0, 0, 0};
                    rc = Vship_ComputeButteraugliYuv(hb, n, nullptr, 0, a.p, a.stride, b.p, b.stride);
                    for (int i = 0; i < 3; i++) scores[3 * l.idx + i] = (float)n[i];
                }
                if (rc != Vship_NoError) {
                    std::cerr << err_text(rc) << "\n";
                    failed = 1;
                }
                const int d = ++done;
                std::lock_guard<std::mutex> lk(out_mu);
                if (o.live) {
                    std::cout << std::setprecision(9) << jobs[l.idx].src_frame;
                    for (int i = 0; i < nres; i++) std::cout << " " << scores[(size_t)nres * l.idx + i];
                    std::cout << "\n";
                } else if (d % 16 == 0 || d == nframes) {
                    std::cout << "\r" << d << "/" << nframes << std::flush;
                }
            }
            if (o.metric == Metric::SSIMU2) Vship_SSIMU2Free(hs);
            else Vship_ButteraugliFree(hb);
        });
    for (auto& t : readers) t.join();
    for (auto& t : workers) t.join();
    if (failed) {
        std::cerr << "A frame worker returned an error, some frames failed to compute\n";
        return 1;
    }
    const double ms = std::chrono::duration<double, std::milli>(std::chrono::high_resolution_clock::now() - t0).count();
    if (!o.json.empty()) {  // doc/FFVship.md: [[s0], [s1], ...] or [[q, 3, inf], ...]
        std::ofstream f(o.json);
        if (!f) {
            std::cerr << "Failed to open output file\n";
            return 1;
        }
        f << std::setprecision(9) << "[";
        for (int i = 0; i < nframes; i++) {
            f << "[";
            for (int k = 0; k < nres; k++) f << scores[(size_t)nres * i + k] << (k + 1 < nres ? ", " : "");
            f << (i + 1 < nframes ? "], " : "]");
        }
        f << "]";
    }
    if (o.live) return 0;
    std::cout << "\n" << (o.metric == Metric::Butteraugli ? "Butteraugli" : "SSIMU2") << " Result between "
              << o.source << " and " << o.encoded << "\n";
    std::cout << "Computed " << nframes << " frames at " << (ms > 0 ? nframes * 1000.0 / ms : 0.0) << " fps\n\n";
    if (o.metric == Metric::Butteraugli) {
        std::vector<float> q(nframes), t3(nframes), inf(nframes);
        for (int i = 0; i < nframes; i++) {
            q[i] = scores[3 * i];
            t3[i] = scores[3 * i + 1];
            inf[i] = scores[3 * i + 2];
        }
        print_stats(q, std::to_string(o.qnorm) + "-Norm");
        print_stats(t3, "3-Norm");
        print_stats(inf, "INF-Norm");
    } else {
        print_stats(scores, "SSIMULACRA2");
    }
    return 0;
}
