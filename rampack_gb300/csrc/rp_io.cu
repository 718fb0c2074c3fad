// Snapshot and trajectory files of a packing, written from device state.
//
// RAMSNAP (text; core/io/RamsnapWriter.cpp:8-48, core/io/RamsnapReader.cpp:16-96) and
// RAMTRJ (binary; core/io/RamtrjIO.cpp:16-101, core/io/RamtrjRecorder.cpp:9-67,
// core/io/RamtrjPlayer.cpp:11-86).  Both formats are the reference's byte for byte:
//   * a RAMSNAP number is what `operator<<` prints at precision max_digits10 (17) in
//     defaultfloat, i.e. printf's %.17g, here produced by std::to_chars (general, 17),
//     which the C++ standard defines as that printf conversion; numbers are read back with
//     the istream grammar (sign, digits, point, exponent) and strtod's correctly rounded
//     conversion, so a written state reads back bit for bit;
//   * a RAMTRJ particle is its position and the first Euler-angle solution of its
//     orientation (geometry/EulerAngles.cpp:12-46), computed on the host with the C
//     library's asin, cos and atan2 in the reference's order, and turned back into a
//     matrix with Matrix::rotation(ax, ay, az) (geometry/Matrix.tpp:411-434).
// A recording from a handle is asynchronous: the device copies its state into a snapshot
// buffer in order with the handle's moves, a side stream downloads it into pinned memory,
// and a writer thread converts and appends it while the handle keeps sweeping.

#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cerrno>
#include <charconv>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "rampack_gb300.h"
#include "rp_geom.cuh"

namespace rp {
int state_snapshot(void *handle, double *pos, double *rot, double *box9, int64_t *n, cudaStream_t side,
                   cudaEvent_t done, std::string &err);
int64_t handle_size(void *handle);
}  // namespace rp

namespace {

thread_local std::string io_error;

int io_fail(int code, const std::string &msg) {
    io_error = msg;
    return code;
}

int host_threads() {
    unsigned t = std::thread::hardware_concurrency();
    return static_cast<int>(std::max(1u, std::min(t, 64u)));
}

// Runs body(begin, end) over [0, n) split into contiguous chunks on several threads.
template <class F>
void parallel_chunks(int64_t n, int64_t min_chunk, F body) {
    const int64_t want = std::max<int64_t>(1, std::min<int64_t>(host_threads(), n / std::max<int64_t>(1, min_chunk)));
    if (want <= 1) {
        body(int64_t{0}, n);
        return;
    }
    std::vector<std::thread> th;
    for (int64_t t = 0; t < want; t++) {
        const int64_t b = n * t / want, e = n * (t + 1) / want;
        th.emplace_back([=] { body(b, e); });
    }
    for (auto &x : th) x.join();
}

// ---- RAMSNAP ----------------------------------------------------------------------

// operator<< of a double with precision 17 and defaultfloat (printf %.17g)
inline char *put_number(char *p, char *end, double v) { return std::to_chars(p, end, v, std::chars_format::general, 17).ptr; }

constexpr int NUMBER_CHARS = 26;  // the longest %.17g: sign, 17 digits, point, "e-308"

bool has_space(const char *s) {
    for (; *s; s++)
        if (std::isspace(static_cast<unsigned char>(*s))) return true;
    return false;
}

// RamsnapWriter::write (core/io/RamsnapWriter.cpp:8-48) of a state held on the host.
int write_ramsnap(const char *path, int64_t n, const double *pos, const double *rot, const double *box9, int32_t naux,
                  const char *const *keys, const char *const *values) {
    if (!path || (n > 0 && (!pos || !rot)) || !box9 || n < 0 || naux < 0 || (naux > 0 && (!keys || !values)))
        return io_fail(RP_ERR_ARG, "null argument");
    // storeAuxInfo: a std::map, so keys in byte order and a repeated key keeps its last value
    std::map<std::string, std::string> aux;
    for (int32_t i = 0; i < naux; i++) {
        if (!keys[i] || !values[i]) return io_fail(RP_ERR_ARG, "null aux entry");
        if (has_space(keys[i])) return io_fail(RP_ERR_ARG, "an aux key contains whitespace");
        aux[keys[i]] = values[i];
    }
    std::string head = std::to_string(aux.size()) + "\n";
    for (auto &kv : aux) head += kv.first + " " + kv.second + "\n";
    // storeBox: the 9 entries row by row, one space apart
    char buf[16 * NUMBER_CHARS];
    char *p = buf;
    for (int k = 0; k < 9; k++) {
        p = put_number(p, buf + sizeof(buf), box9[k]);
        *p++ = k < 8 ? ' ' : '\n';
    }
    head.append(buf, p);
    head += std::to_string(n) + "\n";
    // storeShapes: "x y z" + 8 spaces + the 9 orientation entries, one line per shape
    const int threads = host_threads();
    std::vector<std::string> parts(threads);
    const int64_t per = (n + threads - 1) / std::max(1, threads);
    std::vector<std::thread> th;
    for (int t = 0; t < threads; t++) {
        const int64_t b = std::min<int64_t>(n, t * per), e = std::min<int64_t>(n, (t + 1) * per);
        th.emplace_back([&, t, b, e] {
            std::string &out = parts[t];
            out.resize(static_cast<size_t>((e - b) * (12 * NUMBER_CHARS + 20)));
            char *q = out.data(), *qe = out.data() + out.size();
            for (int64_t i = b; i < e; i++) {
                for (int d = 0; d < 3; d++) {
                    q = put_number(q, qe, pos[3 * i + d]);
                    if (d < 2) *q++ = ' ';
                }
                std::memcpy(q, "        ", 8);
                q += 8;
                for (int k = 0; k < 9; k++) {
                    q = put_number(q, qe, rot[9 * i + k]);
                    *q++ = k < 8 ? ' ' : '\n';
                }
            }
            out.resize(static_cast<size_t>(q - out.data()));
        });
    }
    for (auto &x : th) x.join();
    FILE *f = std::fopen(path, "wb");
    if (!f) return io_fail(RP_ERR_IO, std::string("cannot open ") + path + " for writing");
    bool ok = std::fwrite(head.data(), 1, head.size(), f) == head.size();
    for (auto &s : parts) ok = ok && std::fwrite(s.data(), 1, s.size(), f) == s.size();
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return io_fail(RP_ERR_IO, std::string("write error on ") + path);
    return RP_OK;
}

// The reader's view of a text: std::istream extraction rules over a byte buffer.
struct TextIn {
    const char *p, *end;
    bool ok = true;

    static bool ws(char c) { return c == ' ' || c == '\n' || c == '\t' || c == '\r' || c == '\v' || c == '\f'; }
    void skip_ws() {
        while (p < end && ws(*p)) p++;
    }
    // operator>>(std::size_t): optional '+', decimal digits
    bool read_size(uint64_t &v) {
        skip_ws();
        const char *q = p;
        if (q < end && *q == '+') q++;
        const char *d0 = q;
        uint64_t x = 0;
        while (q < end && *q >= '0' && *q <= '9') {
            const uint64_t d = static_cast<uint64_t>(*q - '0');
            if (x > (UINT64_MAX - d) / 10) return ok = false;
            x = 10 * x + d;
            q++;
        }
        if (q == d0) return ok = false;
        v = x;
        p = q;
        return true;
    }
    // operator>>(std::string): a run of non-whitespace
    bool read_word(std::string &w) {
        skip_ws();
        const char *q = p;
        while (q < end && !ws(*q)) q++;
        if (q == p) return ok = false;
        w.assign(p, q);
        p = q;
        return true;
    }
    // std::getline: up to the next newline, which is consumed
    bool read_line(std::string &l) {
        if (p >= end) return ok = false;
        const char *q = p;
        while (q < end && *q != '\n') q++;
        l.assign(p, q);
        p = q < end ? q + 1 : q;
        return true;
    }
};

// operator>>(double) of libstdc++'s num_get: the longest prefix of the form
// [+-]digits[.digits][(e|E)[+-]digits] is gathered and converted by strtod in the C locale;
// a prefix strtod does not consume whole, or an overflow, fails the stream.
bool parse_number(const char *&p, const char *end, double &v) {
    while (p < end && TextIn::ws(*p)) p++;
    const char *q = p;
    char tok[400];
    int len = 0;
    auto take = [&](char c) {
        if (len < static_cast<int>(sizeof(tok)) - 1) tok[len++] = c;
        q++;
    };
    if (q < end && (*q == '+' || *q == '-')) take(*q);
    bool digits = false;
    while (q < end && *q >= '0' && *q <= '9') {
        take(*q);
        digits = true;
    }
    if (q < end && *q == '.') {
        take(*q);
        while (q < end && *q >= '0' && *q <= '9') {
            take(*q);
            digits = true;
        }
    }
    if (digits && q < end && (*q == 'e' || *q == 'E')) {
        take(*q);
        if (q < end && (*q == '+' || *q == '-')) take(*q);
        while (q < end && *q >= '0' && *q <= '9') take(*q);
    }
    tok[len] = '\0';
    p = q;
    if (!digits || len >= static_cast<int>(sizeof(tok)) - 1) return false;
    double x = 0;
    auto r = std::from_chars(tok, tok + len, x, std::chars_format::general);
    if (r.ec == std::errc() && r.ptr == tok + len && tok[0] != '+') {
        v = x;
        return true;
    }
    // the unusual cases (a leading '+', range errors, a dangling exponent) as strtod sees them
    errno = 0;
    char *e = nullptr;
    x = std::strtod(tok, &e);
    if (e != tok + len) return false;
    if (errno == ERANGE && std::fabs(x) == HUGE_VAL) return false;
    v = x;
    return true;
}

struct Ramsnap {
    std::vector<std::pair<std::string, std::string>> aux;
    double box[9]{};
    std::vector<double> pos, rot;
    int64_t n = 0;
};

// RamsnapReader::read (core/io/RamsnapReader.cpp:16-96).
int read_ramsnap(const char *path, Ramsnap &s) {
    if (!path) return io_fail(RP_ERR_ARG, "null path");
    FILE *f = std::fopen(path, "rb");
    if (!f) return io_fail(RP_ERR_IO, std::string("cannot open ") + path);
    std::string text;
    char chunk[1 << 16];
    size_t got;
    while ((got = std::fread(chunk, 1, sizeof(chunk), f)) > 0) text.append(chunk, got);
    std::fclose(f);
    TextIn in{text.data(), text.data() + text.size()};
    // restoreAuxInfo
    uint64_t naux = 0;
    if (!in.read_size(naux)) return io_fail(RP_ERR_FORMAT, "Broken RAMSNAP file: aux info size");
    std::map<std::string, std::string> aux;
    for (uint64_t i = 0; i < naux; i++) {
        std::string key, value;
        bool ok = in.read_word(key);
        if (ok) {
            in.skip_ws();  // >> std::ws
            ok = in.read_line(value);
        }
        if (!ok) return io_fail(RP_ERR_FORMAT, "Broken RAMSNAP file: aux info entry " + std::to_string(i));
        aux[key] = value;
    }
    s.aux.assign(aux.begin(), aux.end());
    // restoreBox: the rest of the current line holds 3 (old format: the sides of a
    // cuboid) or 9 numbers
    std::string line;
    if (!in.read_line(line)) return io_fail(RP_ERR_FORMAT, "Broken RAMSNAP file: dimensions");
    const char *lp = line.data(), *le = line.data() + line.size();
    double t[9]{};
    for (int k = 0; k < 3; k++)
        if (!parse_number(lp, le, t[k])) return io_fail(RP_ERR_FORMAT, "Broken RAMSNAP file: dimensions");
    const char *rest = lp;
    while (rest < le && TextIn::ws(*rest)) rest++;
    for (double &b : s.box) b = 0.0;
    if (rest == le) {
        s.box[0] = t[0];
        s.box[4] = t[1];
        s.box[8] = t[2];
    } else {
        for (int k = 3; k < 9; k++)
            if (!parse_number(lp, le, t[k])) return io_fail(RP_ERR_FORMAT, "Broken RAMSNAP file: dimensions");
        std::memcpy(s.box, t, sizeof(t));
    }
    // TriclinicBox(dimensions) inverts the matrix (geometry/Matrix.tpp:261-271), then the
    // reader checks TriclinicBox::getVolume (core/TriclinicBox.cpp:35-38): |(s0 x s1) . s2|
    if (rp::det3(s.box) == 0) return io_fail(RP_ERR_FORMAT, "cannot invert, det == 0");
    {
        const double *m = s.box;
        const rp::d3 s0{m[0], m[3], m[6]}, s1{m[1], m[4], m[7]}, s2{m[2], m[5], m[8]};
        if (std::fabs(rp::dot3(rp::cross3(s0, s1), s2)) == 0)
            return io_fail(RP_ERR_FORMAT, "Broken RAMSNAP file: zero box volume");
    }
    // restoreShapes: the token positions are found in one pass, converted in parallel
    uint64_t size = 0;
    if (!in.read_size(size)) return io_fail(RP_ERR_FORMAT, "Broken RAMSNAP file: size");
    if (size > (uint64_t{1} << 40)) return io_fail(RP_ERR_FORMAT, "Broken RAMSNAP file: size");
    s.n = static_cast<int64_t>(size);
    std::vector<const char *> starts(static_cast<size_t>(12 * size + 1));
    {
        const char *q = in.p;
        for (uint64_t k = 0; k < 12 * size; k++) {
            while (q < in.end && TextIn::ws(*q)) q++;
            starts[k] = q;
            while (q < in.end && !TextIn::ws(*q)) q++;
        }
    }
    s.pos.assign(3 * size, 0.0);
    s.rot.assign(9 * size, 0.0);
    std::mutex mu;
    int64_t first_bad = -1;
    parallel_chunks(s.n, 4096, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            for (int k = 0; k < 12; k++) {
                const char *tp = starts[12 * i + k];
                double v = 0;
                // a token is read up to the next whitespace by the scan; the number must be
                // its whole (operator>> stops inside a token, and the next read then fails)
                const char *te = tp;
                while (te < in.end && !TextIn::ws(*te)) te++;
                const char *pp = tp;
                if (tp >= in.end || !parse_number(pp, te, v) || pp != te) {
                    std::lock_guard<std::mutex> lk(mu);
                    if (first_bad < 0 || i < first_bad) first_bad = i;
                    return;
                }
                if (k < 3) s.pos[3 * i + k] = v;
                else s.rot[9 * i + k - 3] = v;
            }
        }
    });
    if (first_bad >= 0)
        return io_fail(RP_ERR_FORMAT, "Broken RAMSNAP file: shape " + std::to_string(first_bad) + "/" +
                                          std::to_string(size));
    return RP_OK;
}

// ---- RAMTRJ -----------------------------------------------------------------------

constexpr int64_t TRJ_HEADER = 7 + 1 + 1 + 8 + 8 + 8;  // RamtrjIO::getHeaderSize

struct TrjHeader {
    uint8_t minor = 1, major = 1;
    uint64_t particles = 0, snapshots = 0, cycle_step = 0;
};

constexpr double PI = 3.14159265358979323846;  // M_PI

int64_t trj_snapshot_bytes(uint64_t particles) { return 9 * 8 + static_cast<int64_t>(particles) * 6 * 8; }

void put_header(const TrjHeader &h, unsigned char out[TRJ_HEADER]) {
    std::memcpy(out, "RAMTRJ\n", 7);
    out[7] = h.minor;  // RamtrjIO::writeHeader: the minor version first
    out[8] = h.major;
    std::memcpy(out + 9, &h.particles, 8);
    std::memcpy(out + 17, &h.snapshots, 8);
    std::memcpy(out + 25, &h.cycle_step, 8);
}

// RamtrjIO::readHeader (core/io/RamtrjIO.cpp:16-38)
int get_header(FILE *f, TrjHeader &h) {
    unsigned char b[TRJ_HEADER];
    if (std::fseek(f, 0, SEEK_SET) != 0 || std::fread(b, 1, 7, f) != 7 || std::memcmp(b, "RAMTRJ\n", 7) != 0)
        return io_fail(RP_ERR_FORMAT, "RAMTRJ read error: magic");
    if (std::fread(b + 7, 1, 2, f) != 2) return io_fail(RP_ERR_FORMAT, "RAMTRJ: only versions up to 1.1 are supported");
    h.minor = b[7];
    h.major = b[8];
    if (!(h.major == 1 && h.minor <= 1)) return io_fail(RP_ERR_FORMAT, "RAMTRJ: only versions up to 1.1 are supported");
    if (std::fread(&h.particles, 8, 1, f) != 1) return io_fail(RP_ERR_FORMAT, "RAMTRJ read error: num particles");
    if (std::fread(&h.snapshots, 8, 1, f) != 1) return io_fail(RP_ERR_FORMAT, "RAMTRJ read error: num snapshots");
    if (std::fread(&h.cycle_step, 8, 1, f) != 1) return io_fail(RP_ERR_FORMAT, "RAMTRJ read error: cycle step");
    if (h.major >= 1 && h.minor >= 1) {
        if (h.particles == 0) return io_fail(RP_ERR_FORMAT, "RAMTRJ read error: num particles");
        if (h.cycle_step == 0) return io_fail(RP_ERR_FORMAT, "RAMTRJ read error: cycle step");
    }
    return RP_OK;
}

int64_t file_size(FILE *f) {
    if (std::fseek(f, 0, SEEK_END) != 0) return -1;
    long s = std::ftell(f);
    return s;
}

// EulerAngles (geometry/EulerAngles.cpp:12-63): the rotation check O·Oᵀ − I within 1e-12
// (Matrix products accumulate from zero in index order, geometry/Matrix.tpp:104-113) and
// the first solution (psi, theta, phi).
bool euler_first(const double *o, double out[3]) {
    constexpr double EPS = 1e-12;
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++) {
            double s = 0.0;
            for (int k = 0; k < 3; k++) s += o[3 * i + k] * o[3 * j + k];
            const double z = s - (i == j ? 1.0 : 0.0);
            if (!(std::fabs(z) < EPS)) return false;
        }
    const double R11 = o[0], R12 = o[1], R13 = o[2], R21 = o[3], R31 = o[6], R32 = o[7], R33 = o[8];
    double psi, theta, phi;
    if (R31 > -1 + EPS || R31 < 1 - EPS) {  // the reference's condition (always true for |R31| <= 1)
        theta = -std::asin(R31);
        const double c1 = std::cos(theta);
        psi = std::atan2(R32 / c1, R33 / c1);
        phi = std::atan2(R21 / c1, R11 / c1);
    } else {
        phi = 0;
        if (R31 < 0) {
            theta = PI / 2;
            psi = std::atan2(R12, R13);
        } else {
            theta = -PI / 2;
            psi = std::atan2(-R12, -R13);
        }
    }
    out[0] = psi;
    out[1] = theta;
    out[2] = phi;
    return true;
}

// Matrix<3,3>::rotation(ax, ay, az) (geometry/Matrix.tpp:411-434)
void euler_matrix(const double a[3], double *m) {
    const double sx = std::sin(a[0]), sy = std::sin(a[1]), sz = std::sin(a[2]);
    const double cx = std::cos(a[0]), cy = std::cos(a[1]), cz = std::cos(a[2]);
    m[0] = cy * cz;
    m[1] = sx * sy * cz - cx * sz;
    m[2] = cx * sy * cz + sx * sz;
    m[3] = cy * sz;
    m[4] = sx * sy * sz + cx * cz;
    m[5] = cx * sy * sz - sx * cz;
    m[6] = -sy;
    m[7] = sx * cy;
    m[8] = cx * cy;
}

// One snapshot's bytes: the box, then position and Euler angles per particle.  Returns
// the first particle whose orientation is not a rotation, or -1.
int64_t encode_snapshot(int64_t n, const double *pos, const double *rot, const double *box9, std::vector<double> &out) {
    out.resize(static_cast<size_t>(9 + 6 * n));
    std::memcpy(out.data(), box9, 9 * sizeof(double));
    std::mutex mu;
    int64_t bad = -1;
    parallel_chunks(n, 8192, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            double *q = out.data() + 9 + 6 * i;
            q[0] = pos[3 * i];
            q[1] = pos[3 * i + 1];
            q[2] = pos[3 * i + 2];
            if (!euler_first(rot + 9 * i, q + 3)) {
                std::lock_guard<std::mutex> lk(mu);
                if (bad < 0 || i < bad) bad = i;
            }
        }
    });
    return bad;
}

// RamtrjRecorder with an asynchronous writer: one snapshot may be in flight (downloading
// or being encoded and written) while the caller goes on.
struct Recorder {
    FILE *f = nullptr;
    TrjHeader h;
    int64_t n = 0;
    // in-flight snapshot
    std::thread worker;
    bool pending = false;
    int pending_rc = RP_OK;
    std::string pending_err;
    double *hpos = nullptr, *hrot = nullptr;  // pinned download buffers
    double box[9]{};
    cudaStream_t side = nullptr;
    cudaEvent_t done = nullptr;
    int device = -1;
    std::string err;

    int wait() {
        if (worker.joinable()) worker.join();
        pending = false;
        if (pending_rc != RP_OK) {
            err = pending_err;
            int rc = pending_rc;
            pending_rc = RP_OK;
            return rc;
        }
        return RP_OK;
    }
    // appends one snapshot (host arrays) and bumps the count
    int append(const double *pos, const double *rot, const double *box9, std::string &e) {
        std::vector<double> buf;
        int64_t bad = encode_snapshot(n, pos, rot, box9, buf);
        if (bad >= 0) {
            e = "orientation of particle " + std::to_string(bad) + " is not a rotation matrix (EulerAngles)";
            return RP_ERR_ARG;
        }
        if (std::fseek(f, 0, SEEK_END) != 0 || std::fwrite(buf.data(), sizeof(double), buf.size(), f) != buf.size() ||
            std::fflush(f) != 0) {
            e = "RAMTRJ write error: snapshot data";
            return RP_ERR_IO;
        }
        h.snapshots++;
        return RP_OK;
    }
};

int recorder_fail(Recorder *r, int code, const std::string &msg) {
    if (r) r->err = msg;
    return io_fail(code, msg);
}

// RamtrjRecorder::recordSnapshot's preconditions (core/io/RamtrjRecorder.cpp:43-47)
int check_cycle(Recorder *r, int64_t cycle) {
    if (cycle <= 0) return recorder_fail(r, RP_ERR_ARG, "cycle must be positive");
    if (static_cast<uint64_t>(cycle) != (r->h.snapshots + (r->pending ? 1 : 0) + 1) * r->h.cycle_step)
        return recorder_fail(r, RP_ERR_ARG, "cycle must be (number of recorded snapshots + 1) * cycle step");
    return RP_OK;
}

}  // namespace

extern "C" {

const char *rp_io_last_error(void) { return io_error.c_str(); }

int rp_ramsnap_write_host(const char *path, int64_t n, const double *pos, const double *rot, const double *box9,
                          int32_t naux, const char *const *keys, const char *const *values) {
    return write_ramsnap(path, n, pos, rot, box9, naux, keys, values);
}

int rp_ramsnap_write(void *handle, const char *path, int32_t naux, const char *const *keys, const char *const *values) {
    if (!handle) return io_fail(RP_ERR_ARG, "null handle");
    const int64_t n = rp::handle_size(handle);
    double *pos = nullptr, *rot = nullptr, box[9];
    if (cudaMallocHost(&pos, sizeof(double) * 3 * std::max<int64_t>(1, n)) != cudaSuccess ||
        cudaMallocHost(&rot, sizeof(double) * 9 * std::max<int64_t>(1, n)) != cudaSuccess) {
        cudaFreeHost(pos);
        return io_fail(RP_ERR_CUDA, "cudaMallocHost failed");
    }
    cudaStream_t side = nullptr;
    cudaEvent_t done = nullptr;
    std::string err;
    int64_t got = 0;
    int rc = RP_OK;
    if (cudaStreamCreateWithFlags(&side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&done, cudaEventDisableTiming) != cudaSuccess) {
        rc = io_fail(RP_ERR_CUDA, "stream or event creation failed");
    } else {
        rc = rp::state_snapshot(handle, pos, rot, box, &got, side, done, err);
        if (rc) io_fail(rc, err);
        else if (cudaEventSynchronize(done) != cudaSuccess) rc = io_fail(RP_ERR_CUDA, "snapshot download failed");
    }
    if (rc == RP_OK) rc = write_ramsnap(path, got, pos, rot, box, naux, keys, values);
    if (done) cudaEventDestroy(done);
    if (side) cudaStreamDestroy(side);
    cudaFreeHost(pos);
    cudaFreeHost(rot);
    return rc;
}

int rp_ramsnap_load(const char *path, void **snap) {
    if (!snap) return io_fail(RP_ERR_ARG, "null argument");
    *snap = nullptr;
    auto *s = new (std::nothrow) Ramsnap();
    if (!s) return io_fail(RP_ERR_ARG, "out of memory");
    int rc = read_ramsnap(path, *s);
    if (rc) {
        delete s;
        return rc;
    }
    *snap = s;
    return RP_OK;
}

int rp_ramsnap_info(void *snap, int64_t *n, int32_t *naux) {
    auto *s = static_cast<Ramsnap *>(snap);
    if (!s) return io_fail(RP_ERR_ARG, "null snapshot");
    if (n) *n = s->n;
    if (naux) *naux = static_cast<int32_t>(s->aux.size());
    return RP_OK;
}

int rp_ramsnap_get(void *snap, double *pos, double *rot, double *box9) {
    auto *s = static_cast<Ramsnap *>(snap);
    if (!s) return io_fail(RP_ERR_ARG, "null snapshot");
    if (pos && s->n) std::memcpy(pos, s->pos.data(), sizeof(double) * 3 * s->n);
    if (rot && s->n) std::memcpy(rot, s->rot.data(), sizeof(double) * 9 * s->n);
    if (box9) std::memcpy(box9, s->box, sizeof(s->box));
    return RP_OK;
}

int rp_ramsnap_aux(void *snap, int32_t i, const char **key, const char **value) {
    auto *s = static_cast<Ramsnap *>(snap);
    if (!s || i < 0 || i >= static_cast<int32_t>(s->aux.size())) return io_fail(RP_ERR_ARG, "bad aux index");
    if (key) *key = s->aux[i].first.c_str();
    if (value) *value = s->aux[i].second.c_str();
    return RP_OK;
}

int rp_ramsnap_free(void *snap) {
    delete static_cast<Ramsnap *>(snap);
    return RP_OK;
}

int rp_ramtrj_open(const char *path, int64_t num_particles, int64_t cycle_step, int append, void **rec) {
    if (!path || !rec) return io_fail(RP_ERR_ARG, "null argument");
    *rec = nullptr;
    if (num_particles <= 0) return io_fail(RP_ERR_ARG, "number of particles must be positive");
    if (cycle_step <= 0) return io_fail(RP_ERR_ARG, "cycle step must be positive");
    auto *r = new (std::nothrow) Recorder();
    if (!r) return io_fail(RP_ERR_ARG, "out of memory");
    r->n = num_particles;
    auto bail = [&](int code, const std::string &msg) {
        if (r->f) std::fclose(r->f);
        delete r;
        return io_fail(code, msg);
    };
    if (append) {
        // RamtrjRecorder(append = true): the header must match, the file must end after its
        // last whole snapshot (core/io/RamtrjRecorder.cpp:15-27)
        r->f = std::fopen(path, "r+b");
        if (!r->f) return bail(RP_ERR_IO, std::string("cannot open ") + path);
        int rc = get_header(r->f, r->h);
        if (rc) return bail(rc, io_error);
        if (r->h.particles != static_cast<uint64_t>(num_particles) || r->h.cycle_step != static_cast<uint64_t>(cycle_step))
            return bail(RP_ERR_ARG, "RAMTRJ append error: unmatching number of molecules and/or cycle step");
        const int64_t want = TRJ_HEADER + static_cast<int64_t>(r->h.snapshots) * trj_snapshot_bytes(r->h.particles);
        if (file_size(r->f) != want) return bail(RP_ERR_FORMAT, "RAMTRJ append error: broken snapshot structure");
    } else {
        r->f = std::fopen(path, "wb");
        if (!r->f) return bail(RP_ERR_IO, std::string("cannot open ") + path + " for writing");
        r->h.particles = static_cast<uint64_t>(num_particles);
        r->h.cycle_step = static_cast<uint64_t>(cycle_step);
        r->h.snapshots = 0;
        unsigned char b[TRJ_HEADER];
        put_header(r->h, b);
        if (std::fwrite(b, 1, TRJ_HEADER, r->f) != TRJ_HEADER) return bail(RP_ERR_IO, "RAMTRJ write error: header");
    }
    *rec = r;
    return RP_OK;
}

int rp_ramtrj_record_host(void *rec, const double *pos, const double *rot, const double *box9, int64_t cycle) {
    auto *r = static_cast<Recorder *>(rec);
    if (!r || !r->f || !pos || !rot || !box9) return io_fail(RP_ERR_ARG, "null argument");
    int rc = r->wait();
    if (rc) return io_fail(rc, r->err);
    rc = check_cycle(r, cycle);
    if (rc) return rc;
    std::string e;
    rc = r->append(pos, rot, box9, e);
    if (rc) return recorder_fail(r, rc, e);
    return RP_OK;
}

int rp_ramtrj_record(void *rec, void *handle, int64_t cycle) {
    auto *r = static_cast<Recorder *>(rec);
    if (!r || !r->f || !handle) return io_fail(RP_ERR_ARG, "null argument");
    int rc = r->wait();
    if (rc) return io_fail(rc, r->err);
    if (rp::handle_size(handle) != r->n) return recorder_fail(r, RP_ERR_ARG, "the packing's size is not the trajectory's");
    rc = check_cycle(r, cycle);
    if (rc) return rc;
    int dev = 0;
    cudaGetDevice(&dev);
    if (!r->hpos) {
        if (cudaMallocHost(&r->hpos, sizeof(double) * 3 * r->n) != cudaSuccess ||
            cudaMallocHost(&r->hrot, sizeof(double) * 9 * r->n) != cudaSuccess ||
            cudaStreamCreateWithFlags(&r->side, cudaStreamNonBlocking) != cudaSuccess ||
            cudaEventCreateWithFlags(&r->done, cudaEventDisableTiming) != cudaSuccess)
            return recorder_fail(r, RP_ERR_CUDA, "pinned buffers, stream or event creation failed");
        r->device = dev;
    }
    std::string err;
    int64_t got = 0;
    rc = rp::state_snapshot(handle, r->hpos, r->hrot, r->box, &got, r->side, r->done, err);
    if (rc) return recorder_fail(r, rc, err);
    r->pending = true;
    r->worker = std::thread([r] {
        if (cudaEventSynchronize(r->done) != cudaSuccess) {
            r->pending_rc = RP_ERR_CUDA;
            r->pending_err = "snapshot download failed";
            return;
        }
        std::string e;
        int code = r->append(r->hpos, r->hrot, r->box, e);
        if (code) {
            r->pending_rc = code;
            r->pending_err = e;
        }
    });
    return RP_OK;
}

int rp_ramtrj_flush(void *rec) {
    auto *r = static_cast<Recorder *>(rec);
    if (!r) return io_fail(RP_ERR_ARG, "null recorder");
    int rc = r->wait();
    if (rc) return io_fail(rc, r->err);
    return RP_OK;
}

int rp_ramtrj_snapshots(void *rec, int64_t *count) {
    auto *r = static_cast<Recorder *>(rec);
    if (!r || !count) return io_fail(RP_ERR_ARG, "null argument");
    int rc = r->wait();
    if (rc) return io_fail(rc, r->err);
    *count = static_cast<int64_t>(r->h.snapshots);
    return RP_OK;
}

// RamtrjRecorder::close0: the header is rewritten with the number of snapshots
int rp_ramtrj_close(void *rec) {
    auto *r = static_cast<Recorder *>(rec);
    if (!r) return io_fail(RP_ERR_ARG, "null recorder");
    int rc = r->wait();
    std::string first_err = rc ? r->err : "";
    if (r->f) {
        unsigned char b[TRJ_HEADER];
        put_header(r->h, b);
        bool ok = std::fseek(r->f, 0, SEEK_SET) == 0 && std::fwrite(b, 1, TRJ_HEADER, r->f) == TRJ_HEADER;
        ok = (std::fclose(r->f) == 0) && ok;
        if (!ok && !rc) {
            rc = RP_ERR_IO;
            first_err = "RAMTRJ write error: header";
        }
    }
    // CUDA objects exist only after a recording from a handle
    if (r->side) cudaStreamDestroy(r->side);
    if (r->done) cudaEventDestroy(r->done);
    if (r->hpos) cudaFreeHost(r->hpos);
    if (r->hrot) cudaFreeHost(r->hrot);
    delete r;
    if (rc) return io_fail(rc, first_err);
    return RP_OK;
}

int rp_ramtrj_info(const char *path, int64_t *num_particles, int64_t *snapshots, int64_t *cycle_step,
                   int32_t *version) {
    if (!path) return io_fail(RP_ERR_ARG, "null path");
    FILE *f = std::fopen(path, "rb");
    if (!f) return io_fail(RP_ERR_IO, std::string("cannot open ") + path);
    TrjHeader h;
    int rc = get_header(f, h);
    // RamtrjPlayer: the file must end after the header's last snapshot (core/io/RamtrjPlayer.cpp:11-18)
    if (!rc && file_size(f) != TRJ_HEADER + static_cast<int64_t>(h.snapshots) * trj_snapshot_bytes(h.particles))
        rc = io_fail(RP_ERR_FORMAT, "RAMTRJ read error: broken snapshot structure");
    std::fclose(f);
    if (rc) return rc;
    if (num_particles) *num_particles = static_cast<int64_t>(h.particles);
    if (snapshots) *snapshots = static_cast<int64_t>(h.snapshots);
    if (cycle_step) *cycle_step = static_cast<int64_t>(h.cycle_step);
    if (version) *version = 256 * h.major + h.minor;
    return RP_OK;
}

// RamtrjPlayer::jumpToSnapshot + nextSnapshot (core/io/RamtrjPlayer.cpp:54-86); `snapshot`
// counts from 0 (the reference's cycle number is (snapshot + 1) · cycle step)
int rp_ramtrj_read(const char *path, int64_t snapshot, double *pos, double *rot, double *box9) {
    if (!path) return io_fail(RP_ERR_ARG, "null path");
    int64_t n = 0, count = 0;
    int rc = rp_ramtrj_info(path, &n, &count, nullptr, nullptr);
    if (rc) return rc;
    if (snapshot < 0 || snapshot >= count) return io_fail(RP_ERR_ARG, "snapshot index out of range");
    FILE *f = std::fopen(path, "rb");
    if (!f) return io_fail(RP_ERR_IO, std::string("cannot open ") + path);
    std::vector<double> buf(static_cast<size_t>(9 + 6 * n));
    const long off = static_cast<long>(TRJ_HEADER + snapshot * trj_snapshot_bytes(static_cast<uint64_t>(n)));
    bool ok = std::fseek(f, off, SEEK_SET) == 0 && std::fread(buf.data(), sizeof(double), buf.size(), f) == buf.size();
    std::fclose(f);
    if (!ok) return io_fail(RP_ERR_FORMAT, "RAMTRJ read error: snapshot particle data");
    if (box9) std::memcpy(box9, buf.data(), 9 * sizeof(double));
    parallel_chunks(n, 8192, [&](int64_t b, int64_t e) {
        for (int64_t i = b; i < e; i++) {
            const double *q = buf.data() + 9 + 6 * i;
            if (pos) {
                pos[3 * i] = q[0];
                pos[3 * i + 1] = q[1];
                pos[3 * i + 2] = q[2];
            }
            if (rot) euler_matrix(q + 3, rot + 9 * i);
        }
    });
    return RP_OK;
}

}  // extern "C"
