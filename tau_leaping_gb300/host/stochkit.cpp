// stochkit.cpp - StochKit-2 XML model reader and writer (host C++).
//
// Reader semantics follow the reference's StochKitReader
// (tau_leaping/StochKitReader.cpp:22-179) and ReadXMLToMatrixStruct
// (tau_leaping/CSCHostMatrixData.cpp:19-107):
//   * species index = position in <SpeciesList>;
//   * a reaction's <Rate> names a <Parameter> Id (a plain number is also
//     accepted, which the reference rejects);
//   * <Reactants> must exist, <Products> may be absent or empty;
//   * a species id repeated inside one list keeps the last stoichiometry;
//   * NumberOfReactions / NumberOfSpecies must match the lists.
// Unlike the reference, every problem is returned as TL_ERR_PARSE with a
// message instead of exiting.  The XML subset parser is this project's own
// (elements, attributes, text, comments, CDATA, declarations).
#include <cctype>
#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <memory>
#include <sstream>
#include <unordered_map>

#include "../csrc/tl_internal.h"

namespace tl {

namespace {

struct XNode {
    std::string name;
    std::vector<std::pair<std::string, std::string>> attrs;
    std::string text;
    std::vector<std::unique_ptr<XNode>> kids;

    const XNode* child(const char* n) const {
        for (auto& k : kids)
            if (k->name == n) return k.get();
        return nullptr;
    }
    std::vector<const XNode*> children(const char* n) const {
        std::vector<const XNode*> r;
        for (auto& k : kids)
            if (k->name == n) r.push_back(k.get());
        return r;
    }
    const std::string* attr(const char* n) const {
        for (auto& a : attrs)
            if (a.first == n) return &a.second;
        return nullptr;
    }
};

class XmlParser {
public:
    XmlParser(const std::string& s) : s_(s) {}

    bool parse(XNode& root, std::string& err) {
        root.name = "#document";
        std::vector<XNode*> stack{&root};
        while (pos_ < s_.size()) {
            if (s_[pos_] != '<') {
                size_t e = s_.find('<', pos_);
                if (e == std::string::npos) e = s_.size();
                stack.back()->text += unescape(s_.substr(pos_, e - pos_));
                pos_ = e;
                continue;
            }
            if (starts("<!--")) {
                size_t e = s_.find("-->", pos_ + 4);
                if (e == std::string::npos) return fail(err, "unterminated comment");
                pos_ = e + 3;
            } else if (starts("<![CDATA[")) {
                size_t e = s_.find("]]>", pos_ + 9);
                if (e == std::string::npos) return fail(err, "unterminated CDATA");
                stack.back()->text += s_.substr(pos_ + 9, e - pos_ - 9);
                pos_ = e + 3;
            } else if (starts("<?")) {
                size_t e = s_.find("?>", pos_ + 2);
                if (e == std::string::npos) return fail(err, "unterminated declaration");
                pos_ = e + 2;
            } else if (starts("<!")) {
                size_t e = s_.find('>', pos_ + 2);
                if (e == std::string::npos) return fail(err, "unterminated <!");
                pos_ = e + 1;
            } else if (starts("</")) {
                pos_ += 2;
                std::string n = name();
                skip_ws();
                if (pos_ >= s_.size() || s_[pos_] != '>') return fail(err, "bad closing tag");
                ++pos_;
                if (stack.size() < 2 || stack.back()->name != n)
                    return fail(err, "mismatched closing tag </" + n + ">");
                stack.pop_back();
            } else {
                ++pos_;
                auto node = std::make_unique<XNode>();
                node->name = name();
                if (node->name.empty()) return fail(err, "empty element name");
                bool self = false;
                for (;;) {
                    skip_ws();
                    if (pos_ >= s_.size()) return fail(err, "unterminated start tag");
                    if (s_[pos_] == '/') {
                        if (pos_ + 1 >= s_.size() || s_[pos_ + 1] != '>') return fail(err, "bad '/' in tag");
                        self = true;
                        pos_ += 2;
                        break;
                    }
                    if (s_[pos_] == '>') {
                        ++pos_;
                        break;
                    }
                    std::string an = name();
                    if (an.empty()) return fail(err, "bad attribute");
                    skip_ws();
                    if (pos_ >= s_.size() || s_[pos_] != '=') return fail(err, "attribute without value");
                    ++pos_;
                    skip_ws();
                    if (pos_ >= s_.size() || (s_[pos_] != '"' && s_[pos_] != '\''))
                        return fail(err, "unquoted attribute value");
                    const char q = s_[pos_++];
                    size_t e = s_.find(q, pos_);
                    if (e == std::string::npos) return fail(err, "unterminated attribute value");
                    node->attrs.push_back({an, unescape(s_.substr(pos_, e - pos_))});
                    pos_ = e + 1;
                }
                XNode* raw = node.get();
                stack.back()->kids.push_back(std::move(node));
                if (!self) stack.push_back(raw);
            }
        }
        if (stack.size() != 1) return fail(err, "unclosed element <" + stack.back()->name + ">");
        return true;
    }

private:
    bool starts(const char* t) const { return s_.compare(pos_, strlen(t), t) == 0; }
    void skip_ws() {
        while (pos_ < s_.size() && isspace((unsigned char)s_[pos_])) ++pos_;
    }
    std::string name() {
        size_t b = pos_;
        while (pos_ < s_.size()) {
            const char c = s_[pos_];
            if (isalnum((unsigned char)c) || c == '_' || c == '-' || c == ':' || c == '.') ++pos_;
            else break;
        }
        return s_.substr(b, pos_ - b);
    }
    static std::string unescape(const std::string& t) {
        std::string r;
        r.reserve(t.size());
        for (size_t i = 0; i < t.size(); ++i) {
            if (t[i] == '&') {
                size_t e = t.find(';', i);
                if (e != std::string::npos) {
                    const std::string ent = t.substr(i + 1, e - i - 1);
                    const char* rep = ent == "lt" ? "<" : ent == "gt" ? ">" : ent == "amp" ? "&"
                                    : ent == "quot" ? "\"" : ent == "apos" ? "'" : nullptr;
                    if (rep) {
                        r += rep;
                        i = e;
                        continue;
                    }
                }
            }
            r += t[i];
        }
        return r;
    }
    bool fail(std::string& err, const std::string& m) {
        size_t line = 1;
        for (size_t i = 0; i < pos_ && i < s_.size(); ++i) line += s_[i] == '\n';
        err = "XML line " + std::to_string(line) + ": " + m;
        return false;
    }
    const std::string& s_;
    size_t pos_ = 0;
};

std::string trim(const std::string& s) {
    size_t b = 0, e = s.size();
    while (b < e && isspace((unsigned char)s[b])) ++b;
    while (e > b && isspace((unsigned char)s[e - 1])) --e;
    return s.substr(b, e - b);
}

const XNode* need(const XNode* parent, const char* n, std::string& err) {
    const XNode* c = parent ? parent->child(n) : nullptr;
    if (!c) err = std::string("can not find ") + n + " node";
    return c;
}

}  // namespace

tl_status parse_stochkit_file(const char* path, HostModel& h, std::vector<Channel>& ch, std::string& err) {
    std::ifstream in(path, std::ios::binary);
    if (!in) {
        err = std::string("can not open file ") + path;
        return TL_ERR_IO;
    }
    std::stringstream ss;
    ss << in.rdbuf();
    const std::string text = ss.str();
    XNode doc;
    XmlParser xp(text);
    if (!xp.parse(doc, err)) return TL_ERR_PARSE;
    const XNode* model = need(&doc, "Model", err);
    if (!model) return TL_ERR_PARSE;
    const XNode* nr = need(model, "NumberOfReactions", err);
    if (!nr) return TL_ERR_PARSE;
    const XNode* ns = need(model, "NumberOfSpecies", err);
    if (!ns) return TL_ERR_PARSE;
    const long n_reactions = strtol(trim(nr->text).c_str(), nullptr, 10);
    const long n_species = strtol(trim(ns->text).c_str(), nullptr, 10);

    // parameters
    std::unordered_map<std::string, double> params;
    const XNode* plist = need(model, "ParametersList", err);
    if (!plist) return TL_ERR_PARSE;
    for (const XNode* pn : plist->children("Parameter")) {
        const XNode* id = need(pn, "Id", err);
        const XNode* ex = need(pn, "Expression", err);
        if (!id || !ex) return TL_ERR_PARSE;
        params[trim(id->text)] = atof(trim(ex->text).c_str());
    }
    // species (indexed in list order)
    const XNode* slist = need(model, "SpeciesList", err);
    if (!slist) return TL_ERR_PARSE;
    std::unordered_map<std::string, int> sidx;
    h.names.clear();
    h.x0.clear();
    for (const XNode* sn : slist->children("Species")) {
        const XNode* id = need(sn, "Id", err);
        const XNode* ip = need(sn, "InitialPopulation", err);
        if (!id || !ip) return TL_ERR_PARSE;
        const std::string name = trim(id->text);
        const std::string pv = trim(ip->text);
        errno = 0;
        char* endp = nullptr;
        long long v = strtoll(pv.c_str(), &endp, 10);
        if (endp == pv.c_str() || errno == ERANGE) {
            // accept "1e5"-style values as the reference's atoi would not
            v = (long long)atof(pv.c_str());
        }
        auto it = sidx.find(name);
        if (it != sidx.end()) {
            h.x0[(size_t)it->second] = v;  // repeated id: last value wins, index kept
            continue;
        }
        sidx[name] = (int)h.names.size();
        h.names.push_back(name);
        h.x0.push_back(v);
    }
    // reactions
    const XNode* rlist = need(model, "ReactionsList", err);
    if (!rlist) return TL_ERR_PARSE;
    ch.clear();
    for (const XNode* rn : rlist->children("Reaction")) {
        Channel c;
        const XNode* rate = need(rn, "Rate", err);
        if (!rate) return TL_ERR_PARSE;
        const std::string rname = trim(rate->text);
        auto pit = params.find(rname);
        if (pit != params.end()) {
            c.rate = pit->second;
        } else {
            char* endp = nullptr;
            const double v = strtod(rname.c_str(), &endp);
            if (endp == rname.c_str() || *endp) {
                err = "can not find the rate for the reaction " + rname;
                return TL_ERR_PARSE;
            }
            c.rate = v;
        }
        auto read_refs = [&](const XNode* list, std::vector<std::pair<int, int>>& out) -> bool {
            if (!list) return true;
            for (const XNode* sr : list->children("SpeciesReference")) {
                const std::string* id = sr->attr("id");
                const std::string* st = sr->attr("stoichiometry");
                if (!id) {
                    err = "SpeciesReference without id";
                    return false;
                }
                auto si = sidx.find(*id);
                if (si == sidx.end()) {
                    err = "reaction references undeclared species " + *id;
                    return false;
                }
                const int stoich = st ? (int)(int8_t)atoi(st->c_str()) : 1;
                bool replaced = false;
                for (auto& e : out)
                    if (e.first == si->second) {
                        e.second = stoich;
                        replaced = true;
                    }
                if (!replaced) out.push_back({si->second, stoich});
            }
            return true;
        };
        const XNode* re = need(rn, "Reactants", err);
        if (!re) return TL_ERR_PARSE;
        if (!read_refs(re, c.reactants)) return TL_ERR_PARSE;
        if (!read_refs(rn->child("Products"), c.products)) return TL_ERR_PARSE;
        ch.push_back(std::move(c));
    }
    if ((long)ch.size() != n_reactions) {
        err = "NumberOfReactions is " + std::to_string(n_reactions) + " but " + std::to_string(ch.size()) +
              " reactions are listed";
        return TL_ERR_PARSE;
    }
    if ((long)h.names.size() != n_species) {
        err = "NumberOfSpecies is " + std::to_string(n_species) + " but " + std::to_string(h.names.size()) +
              " species are listed";
        return TL_ERR_PARSE;
    }
    h.N = (int)h.names.size();
    channels_to_raw(ch, h);
    return TL_OK;
}

tl_status write_stochkit_file(const char* path, const HostModel& h, const std::vector<Channel>& ch,
                              const char* description, std::string& err) {
    FILE* f = fopen(path, "w");
    if (!f) {
        err = std::string("can not write ") + path;
        return TL_ERR_IO;
    }
    fprintf(f, "<!-- StochKit 2.0 text input format -->\n<Model>\n");
    fprintf(f, "  <Description>%s</Description>\n", description ? description : "tau-leaping model");
    fprintf(f, "  <NumberOfReactions>%d</NumberOfReactions>\n", (int)ch.size());
    fprintf(f, "  <NumberOfSpecies>%d</NumberOfSpecies>\n", h.N);
    fprintf(f, "  <ParametersList>\n");
    for (size_t j = 0; j < ch.size(); ++j)
        fprintf(f, "    <Parameter>\n      <Id>c%zu</Id>\n      <Expression>%.9g</Expression>\n    </Parameter>\n",
                j + 1, ch[j].rate);
    fprintf(f, "  </ParametersList>\n  <ReactionsList>\n");
    for (size_t j = 0; j < ch.size(); ++j) {
        fprintf(f, "    <Reaction>\n      <Id>R%zu</Id>\n      <Type>mass-action</Type>\n      <Rate>c%zu</Rate>\n",
                j + 1, j + 1);
        fprintf(f, "      <Reactants>\n");
        for (auto& r : ch[j].reactants)
            fprintf(f, "        <SpeciesReference id=\"%s\" stoichiometry=\"%d\"/>\n", h.names[(size_t)r.first].c_str(),
                    r.second);
        fprintf(f, "      </Reactants>\n      <Products>\n");
        for (auto& p : ch[j].products)
            fprintf(f, "        <SpeciesReference id=\"%s\" stoichiometry=\"%d\"/>\n", h.names[(size_t)p.first].c_str(),
                    p.second);
        fprintf(f, "      </Products>\n    </Reaction>\n");
    }
    fprintf(f, "  </ReactionsList>\n  <SpeciesList>\n");
    for (int i = 0; i < h.N; ++i)
        fprintf(f,
                "    <Species>\n      <Id>%s</Id>\n      <Description>Species #%d</Description>\n"
                "      <InitialPopulation>%lld</InitialPopulation>\n    </Species>\n",
                h.names[(size_t)i].c_str(), i + 1, (long long)h.x0[(size_t)i]);
    fprintf(f, "  </SpeciesList>\n</Model>\n");
    const bool ok = ferror(f) == 0;
    fclose(f);
    if (!ok) {
        err = std::string("write failed for ") + path;
        return TL_ERR_IO;
    }
    return TL_OK;
}

}  // namespace tl
