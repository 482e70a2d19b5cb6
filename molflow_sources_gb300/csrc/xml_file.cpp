// xml_file.cpp — DEFLATE (RFC 1951), ZIP container and XML DOM for the host-side file reader.
#include "xml_file.h"

#include <cstdio>
#include <cstring>

namespace mfgx {

// ------------------------------------------------------------------ inflate ----
namespace {

struct Bits {
    const uint8_t* p;
    size_t n, pos = 0;   // byte position
    uint32_t buf = 0;
    int cnt = 0;
    bool overrun = false;
    uint32_t get(int k) {   // k bits, least significant first
        while (cnt < k) {
            uint32_t b = 0;
            if (pos < n) b = p[pos++];
            else overrun = true;
            buf |= b << cnt;
            cnt += 8;
        }
        const uint32_t v = buf & ((k == 32) ? 0xffffffffu : ((1u << k) - 1u));
        buf >>= k;
        cnt -= k;
        return v;
    }
    void align() { buf = 0; cnt = 0; }   // drop the rest of the current byte
};

// Canonical Huffman code from code lengths: count of codes per length and the symbols in
// code order; decoded one bit at a time against the first code of each length.
struct Huff {
    uint16_t count[16];
    std::vector<uint16_t> sym;
    bool build(const uint8_t* len, int n) {
        std::memset(count, 0, sizeof count);
        for (int i = 0; i < n; ++i) count[len[i]]++;
        count[0] = 0;
        int left = 1;
        for (int l = 1; l < 16; ++l) {   // over-subscribed sets are invalid
            left <<= 1;
            left -= count[l];
            if (left < 0) return false;
        }
        uint16_t offs[16];
        offs[1] = 0;
        for (int l = 1; l < 15; ++l) offs[l + 1] = uint16_t(offs[l] + count[l]);
        sym.assign(size_t(n), 0);
        for (int i = 0; i < n; ++i)
            if (len[i]) sym[offs[len[i]]++] = uint16_t(i);
        return true;
    }
    int decode(Bits& b) const {
        int code = 0, first = 0, index = 0;
        for (int l = 1; l < 16; ++l) {
            code |= int(b.get(1));
            const int c = count[l];
            if (code - first < c) return sym[size_t(index + code - first)];
            index += c;
            first = (first + c) << 1;
            code <<= 1;
        }
        return -1;
    }
};

const uint16_t kLenBase[29] = {3, 4, 5, 6, 7, 8, 9, 10, 11, 13, 15, 17, 19, 23, 27, 31,
                               35, 43, 51, 59, 67, 83, 99, 115, 131, 163, 195, 227, 258};
const uint8_t kLenExtra[29] = {0, 0, 0, 0, 0, 0, 0, 0, 1, 1, 1, 1, 2, 2, 2, 2, 3, 3, 3, 3, 4, 4, 4, 4, 5, 5, 5, 5, 0};
const uint16_t kDistBase[30] = {1, 2, 3, 4, 5, 7, 9, 13, 17, 25, 33, 49, 65, 97, 129, 193,
                                257, 385, 513, 769, 1025, 1537, 2049, 3073, 4097, 6145, 8193, 12289, 16385, 24577};
const uint8_t kDistExtra[30] = {0, 0, 0, 0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6, 6, 7, 7, 8, 8, 9, 9, 10, 10, 11, 11, 12, 12, 13, 13};

bool inflate_codes(Bits& b, const Huff& lit, const Huff& dist, std::vector<uint8_t>& out, std::string& err) {
    while (true) {
        const int s = lit.decode(b);
        if (s < 0 || b.overrun) { err = "deflate: bad literal/length code"; return false; }
        if (s < 256) { out.push_back(uint8_t(s)); continue; }
        if (s == 256) return true;
        const int li = s - 257;
        if (li >= 29) { err = "deflate: bad length symbol"; return false; }
        const size_t len = kLenBase[li] + b.get(kLenExtra[li]);
        const int ds = dist.decode(b);
        if (ds < 0 || ds >= 30) { err = "deflate: bad distance code"; return false; }
        const size_t d = kDistBase[ds] + b.get(kDistExtra[ds]);
        if (d > out.size()) { err = "deflate: distance beyond the output"; return false; }
        const size_t from = out.size() - d;
        for (size_t k = 0; k < len; ++k) out.push_back(out[from + k]);   // may overlap
    }
}

}  // namespace

bool inflate_raw(const uint8_t* in, size_t n, std::vector<uint8_t>& out, std::string& err) {
    Bits b{in, n};
    Huff fl, fd;
    {   // fixed codes (RFC 1951 3.2.6)
        uint8_t len[288];
        for (int i = 0; i < 144; ++i) len[i] = 8;
        for (int i = 144; i < 256; ++i) len[i] = 9;
        for (int i = 256; i < 280; ++i) len[i] = 7;
        for (int i = 280; i < 288; ++i) len[i] = 8;
        fl.build(len, 288);
        uint8_t dl[30];
        for (int i = 0; i < 30; ++i) dl[i] = 5;
        fd.build(dl, 30);
    }
    bool last = false;
    while (!last) {
        last = b.get(1) != 0;
        const uint32_t type = b.get(2);
        if (type == 0) {   // stored
            b.align();
            if (b.pos + 4 > n) { err = "deflate: truncated stored block"; return false; }
            const uint32_t len = uint32_t(in[b.pos]) | (uint32_t(in[b.pos + 1]) << 8);
            const uint32_t nlen = uint32_t(in[b.pos + 2]) | (uint32_t(in[b.pos + 3]) << 8);
            b.pos += 4;
            if ((len ^ 0xffffu) != nlen || b.pos + len > n) { err = "deflate: bad stored block"; return false; }
            out.insert(out.end(), in + b.pos, in + b.pos + len);
            b.pos += len;
        } else if (type == 1) {
            if (!inflate_codes(b, fl, fd, out, err)) return false;
        } else if (type == 2) {   // dynamic codes
            const int nlen = int(b.get(5)) + 257, ndist = int(b.get(5)) + 1, ncode = int(b.get(4)) + 4;
            if (nlen > 286 || ndist > 30) { err = "deflate: bad code counts"; return false; }
            static const uint8_t order[19] = {16, 17, 18, 0, 8, 7, 9, 6, 10, 5, 11, 4, 12, 3, 13, 2, 14, 1, 15};
            uint8_t cl[19] = {0};
            for (int i = 0; i < ncode; ++i) cl[order[i]] = uint8_t(b.get(3));
            Huff ch;
            if (!ch.build(cl, 19)) { err = "deflate: bad code-length code"; return false; }
            uint8_t len[286 + 30];
            int i = 0;
            while (i < nlen + ndist) {
                const int s = ch.decode(b);
                if (s < 0 || b.overrun) { err = "deflate: bad code length"; return false; }
                if (s < 16) { len[i++] = uint8_t(s); continue; }
                int rep = 0;
                uint8_t v = 0;
                if (s == 16) {
                    if (i == 0) { err = "deflate: repeat without a length"; return false; }
                    v = len[i - 1];
                    rep = 3 + int(b.get(2));
                } else if (s == 17) {
                    rep = 3 + int(b.get(3));
                } else {
                    rep = 11 + int(b.get(7));
                }
                if (i + rep > nlen + ndist) { err = "deflate: code lengths overflow"; return false; }
                while (rep--) len[i++] = v;
            }
            if (len[256] == 0) { err = "deflate: no end-of-block code"; return false; }
            Huff dl, dd;
            if (!dl.build(len, nlen) || !dd.build(len + nlen, ndist)) { err = "deflate: bad Huffman code"; return false; }
            if (!inflate_codes(b, dl, dd, out, err)) return false;
        } else {
            err = "deflate: reserved block type";
            return false;
        }
        if (b.overrun) { err = "deflate: truncated stream"; return false; }
    }
    return true;
}

uint32_t crc32(const uint8_t* p, size_t n) {
    static uint32_t table[256];
    static bool init = false;
    if (!init) {
        for (uint32_t i = 0; i < 256; ++i) {
            uint32_t c = i;
            for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xEDB88320u ^ (c >> 1) : c >> 1;
            table[i] = c;
        }
        init = true;
    }
    uint32_t c = 0xffffffffu;
    for (size_t i = 0; i < n; ++i) c = table[(c ^ p[i]) & 0xff] ^ (c >> 8);
    return c ^ 0xffffffffu;
}

// --------------------------------------------------------------------- zip ----
namespace {
uint32_t u16(const std::vector<uint8_t>& z, size_t o) { return uint32_t(z[o]) | (uint32_t(z[o + 1]) << 8); }
uint32_t u32(const std::vector<uint8_t>& z, size_t o) { return u16(z, o) | (u16(z, o + 2) << 16); }
bool ends_xml(const std::string& s) {
    if (s.size() < 4) return false;
    std::string e = s.substr(s.size() - 4);
    for (char& c : e) c = char(c >= 'A' && c <= 'Z' ? c - 'A' + 'a' : c);
    return e == ".xml";
}
}  // namespace

bool zip_first_xml(const std::vector<uint8_t>& z, std::string& xml, std::string& err) {
    // end of central directory record: the last signature 0x06054b50 within the final 64 KiB + 22 B
    if (z.size() < 22) { err = "zip: file too short"; return false; }
    size_t eocd = std::string::npos;
    const size_t lo = z.size() > 65557 ? z.size() - 65557 : 0;
    for (size_t o = z.size() - 22 + 1; o-- > lo;)
        if (u32(z, o) == 0x06054b50u) { eocd = o; break; }
    if (eocd == std::string::npos) { err = "zip: no end of central directory"; return false; }
    const uint32_t entries = u16(z, eocd + 10);
    size_t cd = u32(z, eocd + 16);
    for (uint32_t e = 0; e < entries; ++e) {
        if (cd + 46 > z.size() || u32(z, cd) != 0x02014b50u) { err = "zip: bad central directory"; return false; }
        const uint32_t method = u16(z, cd + 10), crc = u32(z, cd + 16);
        const size_t csize = u32(z, cd + 20), usize = u32(z, cd + 24);
        const size_t nlen = u16(z, cd + 28), xlen = u16(z, cd + 30), clen = u16(z, cd + 32);
        const size_t loc = u32(z, cd + 42);
        if (cd + 46 + nlen > z.size()) { err = "zip: bad entry name"; return false; }
        const std::string name(reinterpret_cast<const char*>(&z[cd + 46]), nlen);
        cd += 46 + nlen + xlen + clen;
        if (!ends_xml(name)) continue;
        if (loc + 30 > z.size() || u32(z, loc) != 0x04034b50u) { err = "zip: bad local header"; return false; }
        const size_t data = loc + 30 + u16(z, loc + 26) + u16(z, loc + 28);
        if (data + csize > z.size()) { err = "zip: truncated entry " + name; return false; }
        std::vector<uint8_t> out;
        if (method == 0) {
            out.assign(z.begin() + long(data), z.begin() + long(data + csize));
        } else if (method == 8) {
            out.reserve(usize);
            if (!inflate_raw(&z[data], csize, out, err)) return false;
        } else {
            err = "zip: compression method " + std::to_string(method) + " of " + name + " is not supported";
            return false;
        }
        if (out.size() != usize || crc32(out.data(), out.size()) != crc) { err = "zip: size or CRC mismatch in " + name; return false; }
        xml.assign(out.begin(), out.end());
        return true;
    }
    err = "zip: no .xml entry";
    return false;
}

bool read_document(const std::string& path, std::string& xml, std::string& err) {
    FILE* f = std::fopen(path.c_str(), "rb");
    if (!f) { err = "cannot open " + path; return false; }
    std::vector<uint8_t> buf;
    uint8_t chunk[1 << 16];
    size_t k;
    while ((k = std::fread(chunk, 1, sizeof chunk, f)) > 0) buf.insert(buf.end(), chunk, chunk + k);
    std::fclose(f);
    std::string low = path;
    for (char& c : low) c = char(c >= 'A' && c <= 'Z' ? c - 'A' + 'a' : c);
    if (low.size() >= 4 && low.compare(low.size() - 4, 4, ".zip") == 0) return zip_first_xml(buf, xml, err);
    xml.assign(buf.begin(), buf.end());
    return true;
}

// --------------------------------------------------------------------- XML ----
const char* XNode::attr(const char* key) const {
    for (const auto& a : attrs)
        if (a.first == key) return a.second.c_str();
    return nullptr;
}
const XNode* XNode::child(const char* tag) const {
    for (const XNode* k : kids)
        if (k->name == tag) return k;
    return nullptr;
}
std::vector<const XNode*> XNode::children(const char* tag) const {
    std::vector<const XNode*> v;
    for (const XNode* k : kids)
        if (k->name == tag) v.push_back(k);
    return v;
}

namespace {
bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r'; }
bool is_name(char c) { return !is_space(c) && c != '>' && c != '/' && c != '=' && c != '<' && c != '"' && c != '\''; }

void put_utf8(std::string& o, uint32_t cp) {
    if (cp < 0x80) { o += char(cp); }
    else if (cp < 0x800) { o += char(0xC0 | (cp >> 6)); o += char(0x80 | (cp & 0x3F)); }
    else if (cp < 0x10000) { o += char(0xE0 | (cp >> 12)); o += char(0x80 | ((cp >> 6) & 0x3F)); o += char(0x80 | (cp & 0x3F)); }
    else { o += char(0xF0 | (cp >> 18)); o += char(0x80 | ((cp >> 12) & 0x3F)); o += char(0x80 | ((cp >> 6) & 0x3F)); o += char(0x80 | (cp & 0x3F)); }
}

// character data with entity and character references decoded
void decode_into(std::string& o, const char* p, const char* e) {
    while (p < e) {
        if (*p != '&') { o += *p++; continue; }
        const char* semi = static_cast<const char*>(std::memchr(p, ';', size_t(e - p)));
        if (!semi) { o += *p++; continue; }
        const std::string ent(p + 1, semi);
        if (ent == "lt") o += '<';
        else if (ent == "gt") o += '>';
        else if (ent == "amp") o += '&';
        else if (ent == "quot") o += '"';
        else if (ent == "apos") o += '\'';
        else if (!ent.empty() && ent[0] == '#') {
            const uint32_t cp = uint32_t(ent.size() > 1 && (ent[1] == 'x' || ent[1] == 'X') ? std::strtoul(ent.c_str() + 2, nullptr, 16)
                                                                                             : std::strtoul(ent.c_str() + 1, nullptr, 10));
            put_utf8(o, cp);
        } else {
            o.append(p, semi + 1);   // unknown entity: kept as written
        }
        p = semi + 1;
    }
}
}  // namespace

bool XDoc::parse(const std::string& s, std::string& err) {
    pool_.clear();
    root_ = nullptr;
    const char* p = s.data();
    const char* e = p + s.size();
    std::vector<XNode*> stack;
    auto fail = [&](const char* what) {
        err = std::string("xml: ") + what + " at byte " + std::to_string(size_t(p - s.data()));
        return false;
    };
    while (p < e) {
        if (*p != '<') {   // character data
            const char* q = static_cast<const char*>(std::memchr(p, '<', size_t(e - p)));
            if (!q) q = e;
            if (!stack.empty()) decode_into(stack.back()->text, p, q);
            p = q;
            continue;
        }
        if (e - p >= 4 && std::strncmp(p, "<!--", 4) == 0) {
            const char* q = std::strstr(p + 4, "-->");
            if (!q) return fail("unterminated comment");
            p = q + 3;
        } else if (e - p >= 9 && std::strncmp(p, "<![CDATA[", 9) == 0) {
            const char* q = std::strstr(p + 9, "]]>");
            if (!q) return fail("unterminated CDATA");
            if (!stack.empty()) stack.back()->text.append(p + 9, q);
            p = q + 3;
        } else if (e - p >= 2 && (p[1] == '?' || p[1] == '!')) {   // processing instruction, DOCTYPE
            const char* q = static_cast<const char*>(std::memchr(p, '>', size_t(e - p)));
            if (!q) return fail("unterminated declaration");
            p = q + 1;
        } else if (e - p >= 2 && p[1] == '/') {   // end tag
            const char* q = static_cast<const char*>(std::memchr(p, '>', size_t(e - p)));
            if (!q) return fail("unterminated end tag");
            std::string name(p + 2, q);
            while (!name.empty() && is_space(name.back())) name.pop_back();
            if (stack.empty() || stack.back()->name != name) return fail("mismatched end tag");
            stack.pop_back();
            p = q + 1;
        } else {   // start tag
            ++p;
            const char* n0 = p;
            while (p < e && is_name(*p)) ++p;
            pool_.emplace_back();
            XNode* node = &pool_.back();
            node->name.assign(n0, p);
            if (node->name.empty()) return fail("empty element name");
            bool closed = false;
            while (true) {
                while (p < e && is_space(*p)) ++p;
                if (p >= e) return fail("unterminated start tag");
                if (*p == '>') { ++p; break; }
                if (*p == '/') {
                    if (p + 1 >= e || p[1] != '>') return fail("bad empty-element tag");
                    p += 2;
                    closed = true;
                    break;
                }
                const char* a0 = p;
                while (p < e && is_name(*p)) ++p;
                std::string key(a0, p);
                while (p < e && is_space(*p)) ++p;
                if (p >= e || *p != '=' || key.empty()) return fail("bad attribute");
                ++p;
                while (p < e && is_space(*p)) ++p;
                if (p >= e || (*p != '"' && *p != '\'')) return fail("unquoted attribute value");
                const char quote = *p++;
                const char* v0 = p;
                while (p < e && *p != quote) ++p;
                if (p >= e) return fail("unterminated attribute value");
                std::string val;
                decode_into(val, v0, p);
                ++p;
                node->attrs.emplace_back(std::move(key), std::move(val));
            }
            if (stack.empty()) {
                if (root_) return fail("second root element");
                root_ = node;
            } else {
                stack.back()->kids.push_back(node);
            }
            if (!closed) stack.push_back(node);
        }
    }
    if (!stack.empty()) { err = "xml: unterminated element <" + stack.back()->name + ">"; return false; }
    if (!root_) { err = "xml: no root element"; return false; }
    return true;
}

}  // namespace mfgx
