// shim_dom.hpp — the subset of the Xerces-C 3.x DOM API that the reference's
// cpu/InitFuncs.cpp (ReadParameters) and linescan/main.cpp (ReadParameters)
// call, written here so those files compile where they lie without the
// Xerces library (test infrastructure for oracle/_ref; not product code).
//
// What it supports is what those two readers need: XercesDOMParser::parse of
// a well-formed file into elements and text (declarations, comments,
// processing instructions and DOCTYPE skipped, attributes ignored, CDATA
// and the five predefined entities plus numeric character references
// decoded), DOMDocument::getElementsByTagName / getDocumentElement,
// DOMNode::getNodeType / getChildNodes / getTextContent, DOMElement::
// getTagName, and XMLString::transcode / equals / release.  XMLCh is a
// 16-bit unit as in Xerces; transcoding to char keeps code points < 256 and
// writes '?' for the rest.  A malformed file raises XMLException, which the
// readers catch.  Validation (Val_Always) is accepted and not performed:
// without a grammar Xerces reports validity problems only through the error
// handler, which HandlerBase ignores.
#ifndef SRS_ORACLE_XERCES_SHIM_DOM_HPP
#define SRS_ORACLE_XERCES_SHIM_DOM_HPP

#include <cstddef>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

namespace xercesc {

typedef char16_t XMLCh;
typedef std::size_t XMLSize_t;

class XMLString {
 public:
  static XMLCh* transcode(const char* s) {
    std::size_t n = std::strlen(s);
    XMLCh* out = new XMLCh[n + 1];
    for (std::size_t i = 0; i < n; ++i) out[i] = (XMLCh)(unsigned char)s[i];
    out[n] = 0;
    return out;
  }
  static char* transcode(const XMLCh* s) {
    std::size_t n = 0;
    while (s[n]) ++n;
    char* out = new char[n + 1];
    for (std::size_t i = 0; i < n; ++i) out[i] = s[i] < 256 ? (char)s[i] : '?';
    out[n] = 0;
    return out;
  }
  static void release(char** p) {
    delete[] *p;
    *p = nullptr;
  }
  static void release(XMLCh** p) {
    delete[] *p;
    *p = nullptr;
  }
  static bool equals(const XMLCh* a, const XMLCh* b) {
    if (!a || !b) return a == b;
    while (*a && *a == *b) ++a, ++b;
    return *a == *b;
  }
};

class XMLException {
 public:
  explicit XMLException(const std::string& m) : msg_(m.begin(), m.end()) {}
  const XMLCh* getMessage() const { return msg_.c_str(); }

 private:
  std::u16string msg_;
};

class DOMException {
 public:
  const XMLCh* msg = u"DOM error";
};

class DOMNodeList;

class DOMNode {
 public:
  enum NodeType { ELEMENT_NODE = 1, TEXT_NODE = 3 };
  DOMNode(short type, std::u16string data) : type_(type), data_(std::move(data)) {}
  virtual ~DOMNode();
  short getNodeType() const { return type_; }
  DOMNodeList* getChildNodes();
  const XMLCh* getTextContent() {
    text_.clear();
    collect(&text_);
    return text_.c_str();
  }
  std::vector<DOMNode*> children_;

 protected:
  void collect(std::u16string* out) const {
    if (type_ == TEXT_NODE) {
      *out += data_;
      return;
    }
    for (const DOMNode* c : children_) c->collect(out);
  }
  short type_;
  std::u16string data_;  // text of a text node, tag name of an element
  std::u16string text_;
  DOMNodeList* list_ = nullptr;
};

class DOMElement : public DOMNode {
 public:
  explicit DOMElement(std::u16string tag) : DOMNode(ELEMENT_NODE, std::move(tag)) {}
  const XMLCh* getTagName() const { return data_.c_str(); }
};

class DOMNodeList {
 public:
  XMLSize_t getLength() const { return v_.size(); }
  DOMNode* item(XMLSize_t i) const { return i < v_.size() ? v_[i] : nullptr; }
  std::vector<DOMNode*> v_;
};

inline DOMNodeList* DOMNode::getChildNodes() {
  if (!list_) list_ = new DOMNodeList();
  list_->v_ = children_;
  return list_;
}

inline DOMNode::~DOMNode() {
  for (DOMNode* c : children_) delete c;
  delete list_;
}

class DOMDocument {
 public:
  ~DOMDocument() {
    delete root_;
    for (DOMNodeList* l : lists_) delete l;
  }
  DOMElement* getDocumentElement() { return root_; }
  DOMNodeList* getElementsByTagName(const XMLCh* name) {
    DOMNodeList* l = new DOMNodeList();
    lists_.push_back(l);
    if (root_) find(root_, name, l);
    return l;
  }
  DOMElement* root_ = nullptr;

 private:
  static void find(DOMNode* n, const XMLCh* name, DOMNodeList* out) {
    if (n->getNodeType() != DOMNode::ELEMENT_NODE) return;
    DOMElement* e = static_cast<DOMElement*>(n);
    if (XMLString::equals(e->getTagName(), name)) out->v_.push_back(e);
    for (DOMNode* c : n->children_) find(c, name, out);
  }
  std::vector<DOMNodeList*> lists_;
};

class ErrorHandler {
 public:
  virtual ~ErrorHandler() {}
};

class HandlerBase : public ErrorHandler {};

class XMLPlatformUtils {
 public:
  static void Initialize() {}
  static void Terminate() {}
};

class XercesDOMParser {
 public:
  enum ValSchemes { Val_Never, Val_Always, Val_Auto };
  ~XercesDOMParser() { delete doc_; }
  void setValidationScheme(ValSchemes) {}
  void setDoNamespaces(bool) {}
  void setErrorHandler(ErrorHandler*) {}
  DOMDocument* getDocument() { return doc_; }

  void parse(const char* path) {
    std::FILE* f = std::fopen(path, "rb");
    if (!f) throw XMLException(std::string("unable to open ") + path);
    std::string s;
    char buf[65536];
    std::size_t n;
    while ((n = std::fread(buf, 1, sizeof(buf), f)) > 0) s.append(buf, n);
    std::fclose(f);
    delete doc_;
    doc_ = new DOMDocument();
    build(s);
  }

 private:
  static bool starts(const std::string& s, std::size_t i, const char* p) {
    return s.compare(i, std::strlen(p), p) == 0;
  }
  static std::size_t skip_to(const std::string& s, std::size_t i, const char* end) {
    std::size_t k = s.find(end, i);
    if (k == std::string::npos) throw XMLException("unterminated markup");
    return k + std::strlen(end);
  }
  // UTF-8 to 16-bit units with the predefined and numeric references decoded
  static std::u16string text(const std::string& s) {
    std::u16string out;
    for (std::size_t i = 0; i < s.size();) {
      unsigned char c = (unsigned char)s[i];
      if (c == '&') {
        std::size_t k = s.find(';', i);
        if (k == std::string::npos) throw XMLException("bad entity reference");
        std::string e = s.substr(i + 1, k - i - 1);
        unsigned long cp = 0;
        if (e == "amp") cp = '&';
        else if (e == "lt") cp = '<';
        else if (e == "gt") cp = '>';
        else if (e == "quot") cp = '"';
        else if (e == "apos") cp = '\'';
        else if (e.size() > 1 && e[0] == '#')
          cp = (e[1] == 'x') ? std::strtoul(e.c_str() + 2, nullptr, 16) : std::strtoul(e.c_str() + 1, nullptr, 10);
        else throw XMLException("unknown entity &" + e + ";");
        out += (char16_t)(cp < 0x10000 ? cp : '?');
        i = k + 1;
      } else if (c < 0x80) {
        out += (char16_t)c;
        ++i;
      } else {
        int len = c >= 0xF0 ? 4 : c >= 0xE0 ? 3 : 2;
        unsigned long cp = c & (0xFF >> (len + 1));
        for (int q = 1; q < len && i + q < s.size(); ++q) cp = (cp << 6) | ((unsigned char)s[i + q] & 0x3F);
        out += (char16_t)(cp < 0x10000 ? cp : '?');
        i += len;
      }
    }
    return out;
  }

  void build(const std::string& s) {
    std::vector<DOMNode*> stack;
    std::size_t i = 0;
    if (starts(s, 0, "\xEF\xBB\xBF")) i = 3;
    while (i < s.size()) {
      if (s[i] != '<') {
        std::size_t k = s.find('<', i);
        if (k == std::string::npos) k = s.size();
        if (!stack.empty()) stack.back()->children_.push_back(new DOMNode(DOMNode::TEXT_NODE, text(s.substr(i, k - i))));
        i = k;
      } else if (starts(s, i, "<?")) {
        i = skip_to(s, i, "?>");
      } else if (starts(s, i, "<!--")) {
        i = skip_to(s, i, "-->");
      } else if (starts(s, i, "<![CDATA[")) {
        std::size_t k = s.find("]]>", i + 9);
        if (k == std::string::npos) throw XMLException("unterminated CDATA");
        std::u16string t(s.begin() + (long)(i + 9), s.begin() + (long)k);
        if (!stack.empty()) stack.back()->children_.push_back(new DOMNode(DOMNode::TEXT_NODE, t));
        i = k + 3;
      } else if (starts(s, i, "<!")) {  // DOCTYPE, with an optional internal subset
        int depth = 0;
        for (++i; i < s.size(); ++i) {
          if (s[i] == '[') ++depth;
          else if (s[i] == ']') --depth;
          else if (s[i] == '>' && depth <= 0) break;
        }
        if (i >= s.size()) throw XMLException("unterminated declaration");
        ++i;
      } else if (starts(s, i, "</")) {
        std::size_t k = s.find('>', i);
        if (k == std::string::npos) throw XMLException("unterminated end tag");
        std::string name = s.substr(i + 2, k - i - 2);
        while (!name.empty() && std::strchr(" \t\r\n", name.back())) name.pop_back();
        if (stack.empty()) throw XMLException("end tag </" + name + "> without a start tag");
        std::u16string want = static_cast<DOMElement*>(stack.back())->getTagName();
        if (std::u16string(name.begin(), name.end()) != want) throw XMLException("mismatched end tag </" + name + ">");
        stack.pop_back();
        i = k + 1;
      } else {
        std::size_t j = i + 1;
        while (j < s.size() && !std::strchr(" \t\r\n/>", s[j])) ++j;
        std::string name = s.substr(i + 1, j - i - 1);
        if (name.empty()) throw XMLException("empty tag name");
        char quote = 0;
        for (; j < s.size(); ++j) {  // attributes are skipped
          if (quote) {
            if (s[j] == quote) quote = 0;
          } else if (s[j] == '"' || s[j] == '\'') {
            quote = s[j];
          } else if (s[j] == '>') {
            break;
          }
        }
        if (j >= s.size()) throw XMLException("unterminated start tag <" + name + ">");
        bool empty = s[j - 1] == '/';
        DOMElement* e = new DOMElement(std::u16string(name.begin(), name.end()));
        if (stack.empty()) {
          if (doc_->root_) {
            delete e;
            throw XMLException("more than one root element");
          }
          doc_->root_ = e;
        } else {
          stack.back()->children_.push_back(e);
        }
        if (!empty) stack.push_back(e);
        i = j + 1;
      }
    }
    if (!stack.empty()) throw XMLException("unclosed element");
    if (!doc_->root_) throw XMLException("no root element");
  }

  DOMDocument* doc_ = nullptr;
};

}  // namespace xercesc

#endif
