/*
 * VTK XML restart / output pieces without the VTK library (the formats of
 * the reference's Cio_data_vtk::readRestart / writeRestart,
 * io_data_vtk.cpp:20-114 and 231-411).  See include/io_data_vtk.h.
 *
 * Binary data arrays: base64 of a little-endian header and the data.  With
 * compressor="vtkZLibDataCompressor" the header is [nblocks, block size,
 * last block size, compressed size of each block] (UInt32 or UInt64 per
 * header_type) and the blocks are zlib streams; without it, one byte count
 * followed by the raw bytes.
 */
#include "io_data_vtk.h"

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <map>
#include <sstream>

#if defined(__has_include)
#if __has_include(<zlib.h>)
#include <zlib.h>
#define SPHDEM_IO_ZLIB 1
#endif
#endif

namespace {

const char B64[] = "ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz0123456789+/";

std::string b64_encode(const unsigned char *p, size_t n) {
    std::string out;
    out.reserve(4 * ((n + 2) / 3));
    for (size_t i = 0; i < n; i += 3) {
        const unsigned v = (unsigned)p[i] << 16 | (i + 1 < n ? (unsigned)p[i + 1] << 8 : 0u) |
                           (i + 2 < n ? (unsigned)p[i + 2] : 0u);
        out += B64[(v >> 18) & 63];
        out += B64[(v >> 12) & 63];
        out += i + 1 < n ? B64[(v >> 6) & 63] : '=';
        out += i + 2 < n ? B64[v & 63] : '=';
    }
    return out;
}

/* decode the base64 characters of s[from, to) (whitespace skipped) */
std::vector<unsigned char> b64_decode(const std::string &s, size_t from, size_t to) {
    static int tab[256];
    static bool init = false;
    if (!init) {
        for (int &t : tab) t = -1;
        for (int i = 0; i < 64; i++) tab[(unsigned char)B64[i]] = i;
        init = true;
    }
    std::vector<unsigned char> out;
    unsigned acc = 0;
    int bits = 0;
    for (size_t i = from; i < to && i < s.size(); i++) {
        const int v = tab[(unsigned char)s[i]];
        if (v < 0) continue;  /* whitespace and padding */
        acc = acc << 6 | (unsigned)v;
        bits += 6;
        if (bits >= 8) {
            bits -= 8;
            out.push_back((unsigned char)(acc >> bits));
        }
    }
    return out;
}

/* the position just past the k-th base64 character of s at or after from */
size_t skip_b64(const std::string &s, size_t from, size_t k) {
    size_t i = from;
    while (i < s.size() && k > 0) {
        const char ch = s[i++];
        if (ch != ' ' && ch != '\n' && ch != '\r' && ch != '\t') k--;
    }
    return i;
}

std::string attr(const std::string &tag, const std::string &name) {
    const std::string key = " " + name + "=\"";
    const size_t p = tag.find(key);
    if (p == std::string::npos) return "";
    const size_t q = tag.find('"', p + key.size());
    return tag.substr(p + key.size(), q - p - key.size());
}

size_t type_size(const std::string &t) {
    if (t == "Float64" || t == "Int64" || t == "UInt64") return 8;
    if (t == "Float32" || t == "Int32" || t == "UInt32") return 4;
    if (t == "Int16" || t == "UInt16") return 2;
    return 1;
}

/* one DataArray body -> doubles (every numeric type) */
bool decode_array(const std::string &body, const std::string &type, bool compressed, bool header64,
                  std::vector<double> &out, std::string &err) {
    const size_t hb = header64 ? 8 : 4;
    auto rd = [&](const unsigned char *p) -> uint64_t {
        uint64_t v = 0;
        for (size_t k = 0; k < hb; k++) v |= (uint64_t)p[k] << (8 * k);
        return v;
    };
    size_t start = 0;
    while (start < body.size() && (body[start] == ' ' || body[start] == '\n' || body[start] == '\r' ||
                                   body[start] == '\t'))
        start++;
    std::vector<unsigned char> raw;
    if (compressed) {
#ifdef SPHDEM_IO_ZLIB
        const size_t first_chars = 4 * ((hb + 2) / 3);
        std::vector<unsigned char> first = b64_decode(body, start, skip_b64(body, start, first_chars));
        if (first.size() < hb) {
            err = "truncated block header";
            return false;
        }
        const uint64_t nblocks = rd(first.data());
        const size_t hbytes = (3 + nblocks) * hb;
        const size_t hchars = 4 * ((hbytes + 2) / 3);
        const size_t hend = skip_b64(body, start, hchars);
        std::vector<unsigned char> head = b64_decode(body, start, hend);
        if (head.size() < hbytes) {
            err = "truncated block header";
            return false;
        }
        const uint64_t bsize = rd(head.data() + hb), last = rd(head.data() + 2 * hb);
        std::vector<unsigned char> data = b64_decode(body, hend, body.size());
        size_t off = 0;
        for (uint64_t b = 0; b < nblocks; b++) {
            const uint64_t cs = rd(head.data() + (3 + b) * hb);
            uLongf len = (uLongf)((b + 1 == nblocks && last) ? last : bsize);
            const size_t at = raw.size();
            raw.resize(at + len);
            if (off + cs > data.size() || uncompress(raw.data() + at, &len, data.data() + off, (uLong)cs) != Z_OK) {
                err = "corrupt zlib block";
                return false;
            }
            raw.resize(at + len);
            off += cs;
        }
#else
        (void)rd;
        err = "the file is zlib-compressed and the reader was built without zlib";
        return false;
#endif
    } else {
        std::vector<unsigned char> all = b64_decode(body, start, body.size());
        if (all.size() < hb) {
            err = "truncated data header";
            return false;
        }
        const uint64_t nbytes = rd(all.data());
        if (all.size() < hb + nbytes) {
            err = "truncated data";
            return false;
        }
        raw.assign(all.begin() + hb, all.begin() + hb + nbytes);
    }
    const size_t ts = type_size(type);
    const size_t n = raw.size() / ts;
    out.resize(n);
    for (size_t i = 0; i < n; i++) {
        const unsigned char *p = raw.data() + i * ts;
        if (type == "Float64") {
            double v;
            std::memcpy(&v, p, 8);
            out[i] = v;
        } else if (type == "Float32") {
            float v;
            std::memcpy(&v, p, 4);
            out[i] = v;
        } else if (type == "Int32") {
            int32_t v;
            std::memcpy(&v, p, 4);
            out[i] = v;
        } else if (type == "UInt32") {
            uint32_t v;
            std::memcpy(&v, p, 4);
            out[i] = v;
        } else if (type == "Int64") {
            int64_t v;
            std::memcpy(&v, p, 8);
            out[i] = (double)v;
        } else if (type == "UInt64") {
            uint64_t v;
            std::memcpy(&v, p, 8);
            out[i] = (double)v;
        } else if (type == "Int8") {
            out[i] = (double)(int8_t)p[0];
        } else {
            out[i] = p[0];
        }
    }
    return true;
}

/* bytes -> one binary DataArray body */
std::string encode_array(const std::vector<unsigned char> &raw) {
#ifdef SPHDEM_IO_ZLIB
    const size_t BS = 32768;
    std::vector<std::vector<unsigned char> > comp;
    for (size_t i = 0; i < raw.size(); i += BS) {
        const size_t len = std::min(BS, raw.size() - i);
        uLongf cl = compressBound((uLong)len);
        std::vector<unsigned char> c(cl);
        compress(c.data(), &cl, raw.data() + i, (uLong)len);
        c.resize(cl);
        comp.push_back(c);
    }
    std::vector<unsigned char> head;
    auto put = [&](uint32_t v) {
        for (int k = 0; k < 4; k++) head.push_back((unsigned char)(v >> (8 * k)));
    };
    put((uint32_t)comp.size());
    put((uint32_t)BS);
    put((uint32_t)(raw.empty() ? 0 : (raw.size() % BS ? raw.size() % BS : BS)));
    for (auto &c : comp) put((uint32_t)c.size());
    std::vector<unsigned char> body;
    for (auto &c : comp) body.insert(body.end(), c.begin(), c.end());
    return b64_encode(head.data(), head.size()) + b64_encode(body.data(), body.size());
#else
    std::vector<unsigned char> all(4);
    const uint32_t n = (uint32_t)raw.size();
    for (int k = 0; k < 4; k++) all[k] = (unsigned char)(n >> (8 * k));
    all.insert(all.end(), raw.begin(), raw.end());
    return b64_encode(all.data(), all.size());
#endif
}

template <typename T>
std::vector<unsigned char> bytes_of(const std::vector<T> &v) {
    std::vector<unsigned char> out(v.size() * sizeof(T));
    if (!v.empty()) std::memcpy(out.data(), v.data(), out.size());
    return out;
}

std::string data_array(const std::string &name, const std::string &type, int ncomp,
                       const std::vector<unsigned char> &raw) {
    std::ostringstream s;
    s << "        <DataArray type=\"" << type << "\"";
    if (!name.empty()) s << " Name=\"" << name << "\"";
    if (ncomp > 1) s << " NumberOfComponents=\"" << ncomp << "\"";
    s << " format=\"binary\">\n          " << encode_array(raw) << "\n        </DataArray>\n";
    return s.str();
}

const char *compressor_attr() {
#ifdef SPHDEM_IO_ZLIB
    return " compressor=\"vtkZLibDataCompressor\"";
#else
    return "";
#endif
}

std::string piece_name(const std::string &stem, int rank) {
    char buf[32];
    std::snprintf(buf, sizeof buf, "_%d.vtu", rank);
    return stem + buf;
}

std::string stem_of(const std::string &base, const char *kind, int timestep) {
    char buf[32];
    std::snprintf(buf, sizeof buf, "%7.7d", timestep);
    return base + kind + buf;
}

}  // namespace

bool Cio_data_vtk::readPiece(const std::string &path, particleContainer &ps) {
    std::ifstream in(path.c_str(), std::ios::binary);
    if (!in) {
        std::cerr << "cannot open " << path << std::endl;
        return false;
    }
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string xml = ss.str();
    const size_t vf = xml.find("<VTKFile");
    if (vf == std::string::npos) {
        std::cerr << path << ": not a VTK XML file" << std::endl;
        return false;
    }
    const std::string root = xml.substr(vf, xml.find('>', vf) - vf);
    const bool compressed = attr(root, "compressor") == "vtkZLibDataCompressor";
    const bool header64 = attr(root, "header_type") == "UInt64";
    const size_t pc = xml.find("<Piece");
    const int n = std::atoi(attr(xml.substr(pc, xml.find('>', pc) - pc), "NumberOfPoints").c_str());
    std::map<std::string, std::vector<double> > arrays;
    std::vector<double> points;
    const size_t pts_at = xml.find("<Points");
    for (size_t at = xml.find("<DataArray"); at != std::string::npos; at = xml.find("<DataArray", at + 1)) {
        const size_t gt = xml.find('>', at);
        const std::string tag = xml.substr(at, gt - at);
        const size_t end = xml.find("</DataArray>", gt);
        const std::string body = xml.substr(gt + 1, end - gt - 1);
        const std::string name = attr(tag, "Name"), type = attr(tag, "type");
        std::vector<double> vals;
        std::string err;
        if (attr(tag, "format") == "ascii") {
            std::istringstream is(body);
            double v;
            while (is >> v) vals.push_back(v);
        } else if (!decode_array(body, type, compressed, header64, vals, err)) {
            std::cerr << path << ": array " << name << ": " << err << std::endl;
            return false;
        }
        /* the points: the first array inside <Points> (VTK may name it) */
        const bool is_points = pts_at != std::string::npos && at > pts_at && points.empty();
        if (is_points) points = vals;
        else if (!name.empty() && (pts_at == std::string::npos || at < pts_at)) arrays[name] = vals;
    }
    if ((int)points.size() < 3 * n) {
        std::cerr << path << ": no points" << std::endl;
        return false;
    }
    auto sca = [&](const char *k, int i, double dflt) {
        auto it = arrays.find(k);
        return it != arrays.end() && (int)it->second.size() > i ? it->second[i] : dflt;
    };
    auto vec = [&](const char *k, int i, vect &out) {
        auto it = arrays.find(k);
        if (it == arrays.end()) return false;
        const int nc = (int)(it->second.size() / (size_t)std::max(n, 1));
        for (int d = 0; d < NDIM && d < nc; d++) out[d] = it->second[(size_t)i * nc + d];
        return true;
    };
    ps.resize(n);
    for (int i = 0; i < n; i++) {
        Cparticle &p = ps[i];
        for (int d = 0; d < NDIM; d++) p.r[d] = points[3 * (size_t)i + d];
        vec("v", i, p.v);
        if (!vec("vhat", i, p.vhat)) p.vhat = p.v;
        vec("norm1", i, p.norm1);
        vec("norm2", i, p.norm2);
        vec("norm3", i, p.norm3);
        vec("f", i, p.f);
        vec("fdrag", i, p.fdrag);
        p.dens = sca("dens", i, 0.0);
        p.h = sca("h", i, 0.0);
        p.mass = sca("mass", i, 0.0);
        p.dddt = sca("dddt", i, 0.0);
        p.radius = sca("radius", i, 0.0);
        p.iam = (iamTypes)(int)sca("iam", i, 0.0);
        p.tag = (int)sca("tag", i, i + 1);
    }
    return true;
}

bool Cio_data_vtk::writePiece(const std::string &path, const particleContainer &ps, bool float64Points) {
    const size_t n = ps.size();
    std::vector<double> sc(n);
    std::vector<int32_t> iv(n);
    std::vector<double> v3(3 * n);
    std::ostringstream s;
    s << "<?xml version=\"1.0\"?>\n<VTKFile type=\"UnstructuredGrid\" version=\"0.1\" "
         "byte_order=\"LittleEndian\""
      << compressor_attr() << ">\n  <UnstructuredGrid>\n    <Piece NumberOfPoints=\"" << n
      << "\" NumberOfCells=\"0\">\n      <PointData Scalars=\"iam\" Vectors=\"v\" Normals=\"norm1\">\n";
    auto scalar = [&](const char *name, double Cparticle::*m) {
        for (size_t i = 0; i < n; i++) sc[i] = m ? ps[i].*m : 0.0;
        s << data_array(name, "Float64", 1, bytes_of(sc));
    };
    auto vector3 = [&](const char *name, vect Cparticle::*m) {
        for (size_t i = 0; i < n; i++)
            for (int d = 0; d < 3; d++) v3[3 * i + d] = (m && d < NDIM) ? (ps[i].*m)[d] : 0.0;
        s << data_array(name, "Float64", 3, bytes_of(v3));
    };
    scalar("dens", &Cparticle::dens);
    scalar("h", &Cparticle::h);
    scalar("eBForce", nullptr);
    scalar("eViscF", nullptr);
    scalar("eViscB", nullptr);
    scalar("eFF", nullptr);
    scalar("u", nullptr);
    scalar("mass", &Cparticle::mass);
    scalar("colour", nullptr);
    for (size_t i = 0; i < n; i++) iv[i] = (int32_t)ps[i].iam;
    s << data_array("iam", "Int32", 1, bytes_of(iv));
    for (size_t i = 0; i < n; i++) iv[i] = ps[i].tag;
    s << data_array("tag", "Int32", 1, bytes_of(iv));
    vector3("v", &Cparticle::v);
    vector3("vhat", &Cparticle::vhat);
    vector3("vort", nullptr);
    vector3("norm1", &Cparticle::norm1);
    vector3("norm2", &Cparticle::norm2);
    if (NDIM == 3) vector3("norm3", &Cparticle::norm3);
    s << "      </PointData>\n      <Points>\n";
    if (float64Points) {
        for (size_t i = 0; i < n; i++)
            for (int d = 0; d < 3; d++) v3[3 * i + d] = d < NDIM ? ps[i].r[d] : 0.0;
        s << data_array("", "Float64", 3, bytes_of(v3));
    } else {
        std::vector<float> f3(3 * n);
        for (size_t i = 0; i < n; i++)
            for (int d = 0; d < 3; d++) f3[3 * i + d] = d < NDIM ? (float)ps[i].r[d] : 0.f;
        s << data_array("", "Float32", 3, bytes_of(f3));
    }
    s << "      </Points>\n      <Cells>\n";
    const std::vector<unsigned char> none;
    s << data_array("connectivity", "Int32", 1, none) << data_array("offsets", "Int32", 1, none)
      << data_array("types", "UInt8", 1, none);
    s << "      </Cells>\n    </Piece>\n  </UnstructuredGrid>\n</VTKFile>\n";
    std::ofstream out(path.c_str(), std::ios::binary);
    out << s.str();
    return (bool)out;
}

void Cio_data_vtk::writeIndex(const std::string &path, const std::vector<std::string> &pieces, bool float64Points) {
    std::ofstream s(path.c_str());
    s << "<?xml version=\"1.0\"?>\n<VTKFile type=\"PUnstructuredGrid\" version=\"0.1\" "
         "byte_order=\"LittleEndian\""
      << compressor_attr() << ">\n  <PUnstructuredGrid GhostLevel=\"0\">\n"
      << "    <PPointData Scalars=\"iam\" Vectors=\"v\" Normals=\"norm1\">\n";
    for (const char *nm : {"dens", "h", "eBForce", "eViscF", "eViscB", "eFF", "u", "mass", "colour"})
        s << "      <PDataArray type=\"Float64\" Name=\"" << nm << "\"/>\n";
    s << "      <PDataArray type=\"Int32\" Name=\"iam\"/>\n      <PDataArray type=\"Int32\" Name=\"tag\"/>\n";
    for (const char *nm : {"v", "vhat", "vort", "norm1", "norm2", "norm3"}) {
        if (NDIM != 3 && !std::strcmp(nm, "norm3")) continue;
        s << "      <PDataArray type=\"Float64\" Name=\"" << nm << "\" NumberOfComponents=\"3\"/>\n";
    }
    s << "    </PPointData>\n    <PPoints>\n      <PDataArray type=\"" << (float64Points ? "Float64" : "Float32")
      << "\" NumberOfComponents=\"3\"/>\n    </PPoints>\n";
    for (const std::string &p : pieces) {
        const size_t slash = p.find_last_of('/');
        s << "    <Piece Source=\"" << (slash == std::string::npos ? p : p.substr(slash + 1)) << "\"/>\n";
    }
    s << "  </PUnstructuredGrid>\n</VTKFile>\n";
}

void Cio_data_vtk::readRestart(int timestep, particleContainer *outPs, CglobalVars *globals) {
    const std::string piece = piece_name(stem_of(filename, "Restart", timestep), globals ? globals->mpiRank : 0);
    std::cout << "Reading file " << piece << std::endl;
    if (!readPiece(piece, *outPs)) std::exit(-1);
    std::cout << "Found " << outPs->size() << " points in the file..." << std::endl;
}

void Cio_data_vtk::writeRestart(int timestep, particleContainer &ps, CglobalVars *globals) {
    const std::string stem = stem_of(filename, "Restart", timestep);
    const std::string piece = piece_name(stem, globals ? globals->mpiRank : 0);
    writePiece(piece, ps, exactPoints);
    writeIndex(stem + ".pvtu", std::vector<std::string>(1, piece), exactPoints);
}

void Cio_data_vtk::writeOutput(int timestep, particleContainer &ps, CglobalVars *globals) {
    const std::string stem = stem_of(filename, "", timestep);
    const std::string piece = piece_name(stem, globals ? globals->mpiRank : 0);
    writePiece(piece, ps, exactPoints);
    writeIndex(stem + ".pvtu", std::vector<std::string>(1, piece), exactPoints);
}

/* ---- Globals and Domain files ------------------------------------------ */

namespace {

std::string rank_file(const std::string &base, const char *what, int rank) {
    return base + what + std::to_string(rank) + ".dat";
}

/* one data row of a Globals file into g (CioGlobals::myGetLine,
 * ioGlobals.cpp:25-37: the columns it reads, the custom ones not); the row's
 * OutStep, or -1 for a line that is not a row */
int parse_globals_row(const std::string &line, CglobalVars *g) {
    std::istringstream ss(line);
    int step = -1;
    if (!(ss >> step)) return -1;
    double lin1 = 0, wt;
    ss >> g->sphStep >> g->time >> g->linMom[0] >> lin1 >> g->angMom >> g->eKE >> g->eBForce >> g->eElast >>
        g->eElastExact >> g->eViscF >> g->eViscB >> g->eFF >> g->eTotal;
    for (int k = 0; k < 6; k++) ss >> wt; /* wall-clock columns */
    ss >> g->maxV >> g->aveDens >> g->varDens >> g->aveDensFromMass >> g->n >> g->nSph >> g->maxF >> g->maxFF >>
        g->rmsFF >> g->edElastdt >> g->edViscFdt >> g->edFFdt;
    if (NDIM > 1) g->linMom[NDIM > 1 ? 1 : 0] = lin1;
    return step;
}

std::string num(double v) {
    char b[32];
    std::snprintf(b, sizeof b, "%.17g", v);
    return b;
}

const char GLOBALS_HEADER[] =
    "# OutStep SPHStep Time linMomX linMomY angMom KE eBForce eElast eElastExact eViscF eViscB eFF eTotal "
    "wtTotalStep wtTotalForceCalc wtTotalDddtCalc wtTotalReset wtTotalUpdateDomain wtTotalMPI maxV aveDens varDens "
    "aveDensFromMass n nSph maxF maxFF rmsFF edElastdt edViscFdt edFFdt";

}  // namespace

void Cio_data_vtk::readGlobals(int outStep, CglobalVars *g) {
    std::ifstream in(rank_file(filename, "Globals", g->mpiRank).c_str());
    if (!in || outStep <= 0) return; /* ioGlobals.cpp:62: no row for step 0 */
    std::string line;
    std::getline(in, line); /* the header */
    while (std::getline(in, line)) {
        const int step = parse_globals_row(line, g);
        if (step >= outStep) break;
    }
}

void Cio_data_vtk::writeGlobals(int outStep, CglobalVars *g) {
    const std::string path = rank_file(filename, "Globals", g->mpiRank);
    std::vector<std::string> lines;
    {
        std::ifstream in(path.c_str());
        std::string line;
        while (std::getline(in, line)) lines.push_back(line);
    }
    if (lines.empty()) lines.push_back(GLOBALS_HEADER);
    /* the write position of openAndSeekToStep(outStep - 1) (ioGlobals.cpp:48-73):
     * right after the header for outStep - 1 <= 0, after the row of outStep - 1
     * if the rows reach it, else at the end */
    size_t keep = lines.size();
    if (outStep - 1 <= 0) {
        keep = 1;
    } else {
        CglobalVars scratch;
        for (size_t i = 1; i < lines.size(); i++) {
            const int step = parse_globals_row(lines[i], &scratch);
            if (step >= outStep - 1) {
                if (step == outStep - 1) keep = i + 1;
                break;
            }
        }
    }
    lines.resize(keep);
    std::ostringstream row;
    row << outStep << ' ' << g->sphStep << ' ' << num(g->time) << ' ' << num(g->linMom[0]) << ' '
        << num(NDIM > 1 ? g->linMom[NDIM > 1 ? 1 : 0] : 0.0) << ' ' << num(g->angMom) << ' ' << num(g->eKE) << ' '
        << num(g->eBForce) << ' ' << num(g->eElast) << ' ' << num(g->eElastExact) << ' ' << num(g->eViscF) << ' '
        << num(g->eViscB) << ' ' << num(g->eFF) << ' ' << num(g->eTotal);
    for (int k = 0; k < 6; k++) row << " 0"; /* wall-clock columns: not measured here */
    row << ' ' << num(g->maxV) << ' ' << num(g->aveDens) << ' ' << num(g->varDens) << ' ' << num(g->aveDensFromMass)
        << ' ' << g->n << ' ' << g->nSph << ' ' << num(g->maxF) << ' ' << num(g->maxFF) << ' ' << num(g->rmsFF) << ' '
        << num(g->edElastdt) << ' ' << num(g->edViscFdt) << ' ' << num(g->edFFdt);
    for (int k = 0; k < GLOBAL_CUSTOM_BUFFER_SIZE; k++) row << ' ' << num(g->custom[k]);
    lines.push_back(row.str());
    std::ofstream out(path.c_str(), std::ios::trunc);
    for (const std::string &l : lines) out << l << '\n';
}

bool Cio_data_vtk::readDomain(int, CglobalVars *g) {
    std::ifstream in(rank_file(filename, "Domain", g->mpiRank).c_str());
    int rank = 0;
    if (!(in >> rank)) return false;
    for (int i = 0; i < 2 * NDIM; i++)
        if (!(in >> g->procDomain[i])) return false;
    for (int k = 0; k < SPHDEM_FACADE_NEIGHBOURS; k++)
        if (!(in >> g->procNeighbrs[k])) return false;
    g->mpiRank = rank;
    g->procNeighbrs[SPHDEM_FACADE_NEIGHBOURS / 2] = -1; /* the process itself (ioDomain.cpp:14-15) */
    return true;
}

void Cio_data_vtk::writeDomain(int, CglobalVars *g) {
    std::ofstream out(rank_file(filename, "Domain", g->mpiRank).c_str(), std::ios::trunc);
    out << g->mpiRank << ' ';
    for (int i = 0; i < 2 * NDIM; i++) out << num(g->procDomain[i]) << ' ';
    for (int k = 0; k < SPHDEM_FACADE_NEIGHBOURS; k++) out << g->procNeighbrs[k] << ' ';
    out << '\n';
}
