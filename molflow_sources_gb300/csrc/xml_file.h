// xml_file.h — reading MolFlow+ files on the C++ host: the XML document of a .xml file, or of
// the .xml inside a .zip (the reference's own test cases and saved results are .zip files).
// Self-contained: a DEFLATE decoder (RFC 1951), the ZIP container (central directory, stored
// and deflated entries, CRC-32 check) and a small XML DOM (elements, attributes, text, the
// five predefined entities and character references, comments, CDATA, processing
// instructions).
#pragma once
#include <cstdint>
#include <deque>
#include <string>
#include <vector>

namespace mfgx {

// Inflate a raw DEFLATE stream (no zlib header) into `out`; false with `err` on a malformed stream.
bool inflate_raw(const uint8_t* in, size_t n, std::vector<uint8_t>& out, std::string& err);

uint32_t crc32(const uint8_t* p, size_t n);

// The first entry of a ZIP archive whose name ends in ".xml" (any case).
bool zip_first_xml(const std::vector<uint8_t>& zip, std::string& xml, std::string& err);

// Whole file, or for a ".zip" path its first XML entry.
bool read_document(const std::string& path, std::string& xml, std::string& err);

struct XNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<XNode*> kids;
    std::string text;   // character data directly inside the element, entities decoded

    const char* attr(const char* key) const;
    const XNode* child(const char* tag) const;   // first child element with this name
    std::vector<const XNode*> children(const char* tag) const;
};

class XDoc {
public:
    bool parse(const std::string& s, std::string& err);
    const XNode* root() const { return root_; }

private:
    std::deque<XNode> pool_;
    XNode* root_ = nullptr;
};

}  // namespace mfgx
