// Minimal XML document model for VXA / VXD / VXT files: elements, attributes,
// text and CDATA.  Replaces the reference's tinyxml (Voxelyze3/src/old/tinyxml*)
// and Boost.PropertyTree readers; only what VXA files use is supported.
#pragma once
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace gvx {

struct XmlNode {
    std::string tag;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::string text;                                   // concatenated text + CDATA content
    std::vector<std::unique_ptr<XmlNode>> children;

    const XmlNode* child(const std::string& name) const;              // first child with this tag
    XmlNode* child(const std::string& name);
    std::vector<const XmlNode*> children_named(const std::string& name) const;
    const char* attr(const std::string& name) const;                 // nullptr if absent
    const XmlNode* path(const std::string& dotted) const;            // "VXA.Simulator.X" from this node (first part must match tag)
    std::unique_ptr<XmlNode> clone() const;
};

// Parses a document; returns nullptr and fills err on malformed input.
std::unique_ptr<XmlNode> xml_parse(const std::string& src, std::string* err);
// Serialises a node (used for report output and round-trip tests).
std::string xml_write(const XmlNode& n, int indent = 0);
std::string xml_escape(const std::string& s);

}  // namespace gvx
