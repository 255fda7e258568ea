// transio.cc — save and load a spline transformation (checkpoint / resume of
// a registration, the output transformation of the registration programs).
//
// The reference writes C2D/C3DTransformation through boost::serialization
// (mia/3d/transio/serialization.hh:35-83, the `xml` plugin
// mia/3d/transio/xml.cc:55-73, 2D likewise): the creator string, the image
// size per axis (size_x, size_y[, size_z]), the attribute map (name ->
// string) and the parameter vector, in that order.  This file writes the
// same fields in the layout of Boost's XML archive (one element per field;
// the map and the vector as count / item_version / item lists) and reads it
// back; doubles are written with 17 significant digits, so a save / load
// round trip returns the same values.  The coefficient grid, which the
// reference derives from the creator's rate and which refine() changes, is
// kept in the attribute map as "csize" ("nx,ny[,nz]").
#include <cstdio>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mgr.h"

namespace mgr {
void set_last_error(const std::string &msg);
}

namespace {

std::string xml_escape(const std::string &s)
{
    std::string o;
    for (char c : s) {
        switch (c) {
        case '&': o += "&amp;"; break;
        case '<': o += "&lt;"; break;
        case '>': o += "&gt;"; break;
        case '"': o += "&quot;"; break;
        case '\'': o += "&apos;"; break;
        default: o += c;
        }
    }
    return o;
}

std::string xml_unescape(const std::string &s)
{
    std::string o;
    for (size_t i = 0; i < s.size(); ++i) {
        if (s[i] != '&') {
            o += s[i];
            continue;
        }
        static const char *names[][2] = {{"&amp;", "&"}, {"&lt;", "<"}, {"&gt;", ">"}, {"&quot;", "\""}, {"&apos;", "'"}};
        bool done = false;
        for (auto &n : names)
            if (s.compare(i, std::strlen(n[0]), n[0]) == 0) {
                o += n[1];
                i += std::strlen(n[0]) - 1;
                done = true;
                break;
            }
        if (!done) o += '&';
    }
    return o;
}

std::string fmt_double(double v)
{
    char b[40];
    std::snprintf(b, sizeof b, "%.17g", v);
    return b;
}

// a minimal reader of the archive: the text of element `name` at or after
// position `pos` (attributes of the start tag ignored); pos moves past it
bool next_element(const std::string &doc, size_t &pos, const std::string &name, std::string &text)
{
    const std::string open = "<" + name;
    size_t p = pos;
    for (;;) {
        p = doc.find(open, p);
        if (p == std::string::npos) return false;
        const char c = doc[p + open.size()];
        if (c == '>' || c == ' ' || c == '\t' || c == '\n' || c == '/') break;
        p += open.size();
    }
    const size_t gt = doc.find('>', p);
    if (gt == std::string::npos) return false;
    if (doc[gt - 1] == '/') {   // <name/>: empty
        text.clear();
        pos = gt + 1;
        return true;
    }
    const std::string close = "</" + name + ">";
    const size_t end = doc.find(close, gt + 1);
    if (end == std::string::npos) return false;
    text = doc.substr(gt + 1, end - gt - 1);
    pos = end + close.size();
    return true;
}

std::string trim(const std::string &s)
{
    const size_t a = s.find_first_not_of(" \t\r\n"), b = s.find_last_not_of(" \t\r\n");
    return a == std::string::npos ? std::string() : s.substr(a, b - a + 1);
}

struct Transform {
    std::string creator;
    int dim = 0;
    int size[3] = {1, 1, 1};
    std::map<std::string, std::string> attr;
    std::vector<double> params;
};

std::string write_doc(const Transform &t)
{
    static const char *axes[3] = {"size_x", "size_y", "size_z"};
    std::ostringstream o;
    o << "<?xml version=\"1.0\" encoding=\"UTF-8\" standalone=\"yes\" ?>\n"
      << "<!DOCTYPE boost_serialization>\n"
      << "<boost_serialization signature=\"serialization::archive\" version=\"17\">\n";
    o << "<creator>" << xml_escape(t.creator) << "</creator>\n";
    for (int k = 0; k < t.dim; ++k) o << "<" << axes[k] << ">" << t.size[k] << "</" << axes[k] << ">\n";
    o << "<attributes class_id=\"0\" tracking_level=\"0\" version=\"0\">\n"
      << "\t<count>" << t.attr.size() << "</count>\n\t<item_version>0</item_version>\n";
    bool first = true;
    for (auto &kv : t.attr) {
        o << "\t<item" << (first ? " class_id=\"1\" tracking_level=\"0\" version=\"0\"" : "") << ">\n"
          << "\t\t<first>" << xml_escape(kv.first) << "</first>\n"
          << "\t\t<second>" << xml_escape(kv.second) << "</second>\n\t</item>\n";
        first = false;
    }
    o << "</attributes>\n";
    o << "<params>\n\t<count>" << t.params.size() << "</count>\n\t<item_version>0</item_version>\n";
    for (double v : t.params) o << "\t<item>" << fmt_double(v) << "</item>\n";
    o << "</params>\n</boost_serialization>\n\n";
    return o.str();
}

Transform read_doc(const std::string &doc)
{
    Transform t;
    size_t pos = 0;
    std::string s;
    if (doc.find("<boost_serialization") == std::string::npos) throw std::invalid_argument("not a transformation archive");
    if (!next_element(doc, pos, "creator", s)) throw std::invalid_argument("archive: no creator");
    t.creator = xml_unescape(trim(s));
    static const char *axes[3] = {"size_x", "size_y", "size_z"};
    for (int k = 0; k < 3; ++k) {
        size_t p2 = pos;
        if (!next_element(doc, p2, axes[k], s)) break;
        const size_t a = doc.find("<attributes", pos);
        if (a != std::string::npos && p2 > a) break;   // (size_z absent in 2D)
        t.size[k] = std::stoi(trim(s));
        t.dim = k + 1;
        pos = p2;
    }
    if (t.dim < 2) throw std::invalid_argument("archive: image size missing");
    std::string attrs;
    if (!next_element(doc, pos, "attributes", attrs)) throw std::invalid_argument("archive: no attributes");
    {
        size_t p = 0;
        std::string item;
        while (next_element(attrs, p, "item", item)) {
            size_t q = 0;
            std::string k, v;
            if (!next_element(item, q, "first", k) || !next_element(item, q, "second", v))
                throw std::invalid_argument("archive: malformed attribute");
            t.attr[xml_unescape(trim(k))] = xml_unescape(trim(v));
        }
    }
    std::string ps;
    if (!next_element(doc, pos, "params", ps)) throw std::invalid_argument("archive: no params");
    size_t p = 0;
    std::string cnt;
    if (!next_element(ps, p, "count", cnt)) throw std::invalid_argument("archive: params without count");
    const size_t n = std::stoull(trim(cnt));
    t.params.reserve(n);
    std::string item;
    while (next_element(ps, p, "item", item)) t.params.push_back(std::stod(trim(item)));
    if (t.params.size() != n) throw std::invalid_argument("archive: params count mismatch");
    return t;
}

std::string csize_text(int dim, const int csize[3])
{
    std::string s;
    for (int k = 0; k < dim; ++k) s += (k ? "," : "") + std::to_string(csize[k]);
    return s;
}

template <class F>
mgr_status guard(const char *who, F f)
{
    try {
        f();
        return MGR_OK;
    } catch (const std::invalid_argument &e) {
        mgr::set_last_error(std::string(who) + ": " + e.what());
        return MGR_ERR_ARG;
    } catch (const std::exception &e) {
        mgr::set_last_error(std::string(who) + ": " + e.what());
        return MGR_ERR_ARG;
    }
}

}  // namespace

extern "C" mgr_status mgr_transform_save(const char *path, int dim, const int size[3], const int csize[3],
                                         const char *creator, const double *params, size_t nparams,
                                         const char *const *attr_names, const char *const *attr_values,
                                         int nattr)
{
    return guard("mgr_transform_save", [&] {
        if (!path || !size || !csize || !creator || (nparams && !params) || (dim != 2 && dim != 3) || nattr < 0 ||
            (nattr && (!attr_names || !attr_values)))
            throw std::invalid_argument("invalid argument");
        size_t nc = size_t(dim);
        for (int k = 0; k < dim; ++k) {
            if (size[k] < 1 || csize[k] < 1) throw std::invalid_argument("sizes must be positive");
            nc *= size_t(csize[k]);
        }
        if (nc != nparams) throw std::invalid_argument("params must hold prod(csize) * dim values");
        Transform t;
        t.creator = creator;
        t.dim = dim;
        for (int k = 0; k < dim; ++k) t.size[k] = size[k];
        for (int i = 0; i < nattr; ++i) t.attr[attr_names[i]] = attr_values[i];
        t.attr["csize"] = csize_text(dim, csize);
        t.params.assign(params, params + nparams);
        std::ofstream f(path, std::ios::binary);
        if (!f) throw std::runtime_error(std::string("cannot write ") + path);
        f << write_doc(t);
        if (!f.good()) throw std::runtime_error(std::string("write failed: ") + path);
    });
}

extern "C" mgr_status mgr_transform_load(const char *path, int *dim, int size[3], int csize[3], char *creator,
                                         size_t creator_cap, char *attrs, size_t attrs_cap, double *params,
                                         size_t params_cap, size_t *nparams)
{
    return guard("mgr_transform_load", [&] {
        if (!path || !dim || !size || !csize || !nparams) throw std::invalid_argument("invalid argument");
        std::ifstream f(path, std::ios::binary);
        if (!f) throw std::invalid_argument(std::string("cannot read ") + path);
        std::stringstream ss;
        ss << f.rdbuf();
        const Transform t = read_doc(ss.str());
        *dim = t.dim;
        for (int k = 0; k < 3; ++k) size[k] = k < t.dim ? t.size[k] : 1;
        auto it = t.attr.find("csize");
        if (it == t.attr.end()) throw std::invalid_argument("archive: no csize attribute");
        int c[3] = {1, 1, 1};
        {
            std::stringstream cs(it->second);
            std::string tok;
            int k = 0;
            while (std::getline(cs, tok, ',') && k < 3) c[k++] = std::stoi(tok);
            if (k != t.dim) throw std::invalid_argument("archive: csize does not match the dimension");
        }
        size_t nc = size_t(t.dim);
        for (int k = 0; k < t.dim; ++k) nc *= size_t(c[k]);
        if (nc != t.params.size()) throw std::invalid_argument("archive: params do not match csize");
        for (int k = 0; k < 3; ++k) csize[k] = c[k];
        *nparams = t.params.size();
        // strings are copied whole or not at all: a buffer too small is an
        // error that names the size needed
        if (creator && creator_cap) {
            if (t.creator.size() + 1 > creator_cap)
                throw std::invalid_argument("creator buffer too small: " + std::to_string(t.creator.size() + 1) +
                                            " bytes needed");
            std::memcpy(creator, t.creator.c_str(), t.creator.size() + 1);
        }
        if (attrs && attrs_cap) {   // "name\tvalue\n" per attribute other than csize
            std::string a;
            for (auto &kv : t.attr)
                if (kv.first != "csize") a += kv.first + "\t" + kv.second + "\n";
            if (a.size() + 1 > attrs_cap)
                throw std::invalid_argument("attribute buffer too small: " + std::to_string(a.size() + 1) +
                                            " bytes needed");
            std::memcpy(attrs, a.c_str(), a.size() + 1);
        }
        if (params) {
            if (params_cap < t.params.size()) throw std::invalid_argument("params buffer too small");
            std::copy(t.params.begin(), t.params.end(), params);
        }
    });
}
