// Minimal XML element/attribute reader for the OpenMM-style system and state
// files: elements, attributes (single or double quoted, the five predefined
// entities decoded), comments, processing instructions and self-closing tags.
// Text content is skipped; the inputs carry everything in attributes.
#pragma once

#include <memory>
#include <string>
#include <vector>

namespace nxm {

struct XmlNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::vector<std::unique_ptr<XmlNode>> children;

    const XmlNode *child(const char *n) const;
    std::vector<const XmlNode *> children_named(const char *n) const;
    const char *attr(const char *n) const;  // nullptr when absent
    // Attribute conversions with pugixml's conventions: a missing or
    // unparsable attribute reads as 0.
    double as_double(const char *n) const;
    int as_int(const char *n) const;
};

struct XmlDoc {
    XmlNode root;       // synthetic root holding the top-level elements
    std::string error;  // empty when the file parsed
};

// Parse a file; on failure doc.error describes it (position and reason).
XmlDoc xml_load_file(const std::string &path);
XmlDoc xml_parse(const std::string &text);

}  // namespace nxm
