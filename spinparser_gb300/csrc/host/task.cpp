// Task-file parser and status log (see task.hpp).
#include "task.hpp"
#include "error.hpp"
#include "lattice.hpp"
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <functional>
#include <set>
#include <strings.h>
#include <sys/stat.h>

namespace spn {

namespace {

const char *kMonths[12] = {"Jan", "Feb", "Mar", "Apr", "May", "Jun", "Jul", "Aug", "Sep", "Oct", "Nov", "Dec"};

[[noreturn]] void init_error(const std::string &m) { throw Error(ErrorType::Initialization, m); }

bool file_exists(const std::string &p) {
    struct stat st;
    return ::stat(p.c_str(), &st) == 0;
}

// property_tree paths of the reference ("task.parameters.frequency") resolve to the first
// child of each name; a missing element is reported by its dotted path.
const XmlNode *at_path(const XmlNode &root, const std::string &path) {
    const XmlNode *n = &root;
    size_t p = 0;
    while (p <= path.size() && !path.empty()) {
        size_t q = path.find('.', p);
        std::string part = path.substr(p, q == std::string::npos ? std::string::npos : q - p);
        n = n->child(part);
        if (!n) return nullptr;
        if (q == std::string::npos) break;
        p = q + 1;
    }
    return n;
}

std::string join(const std::string &a, const std::string &b) { return a.empty() ? b : a + "." + b; }

// _validateProperties (src/TaskFileParser.cpp:357-395): required and optional children and
// attributes of one element; anything else is an error.
void validate(const XmlNode &root, const std::string &node, const std::set<std::string> &req_children,
              const std::set<std::string> &req_attrs, const std::set<std::string> &opt_children = {},
              const std::set<std::string> &opt_attrs = {}, const std::string &tree_path = "") {
    const XmlNode *n = node.empty() ? &root : at_path(root, node);
    if (!n) init_error("Invalid task file. Missing parameter '" + node + "'.");
    const std::string where = join(tree_path, node);
    for (const auto &c : req_children)
        if (!n->child(c)) init_error("Invalid task file. Missing parameter '" + join(where, c) + "'.");
    for (const auto &a : req_attrs)
        if (!n->attr(a)) init_error("Invalid task file. Missing attribute '" + join(where, a) + "'.");
    std::set<std::string> all_children(req_children);
    all_children.insert(opt_children.begin(), opt_children.end());
    for (const auto &c : n->children)
        if (!all_children.count(c.name)) init_error("Invalid task file. Unknown parameter '" + join(where, c.name) + "'.");
    std::set<std::string> all_attrs(req_attrs);
    all_attrs.insert(opt_attrs.begin(), opt_attrs.end());
    for (const auto &a : n->attrs)
        if (!all_attrs.count(a.first)) init_error("Invalid task file. Unknown attribute '" + join(where, a.first) + "'.");
}

std::string text_of(const XmlNode &root, const std::string &path) {
    const XmlNode *n = at_path(root, path);
    if (!n) init_error("Invalid task file. Missing parameter '" + path + "'.");
    return n->text;
}

float to_float(const std::string &s) { return float(parse_number(s)); }

std::string directory_of(const std::string &path) {
    size_t p = path.find_last_of('/');
    return p == std::string::npos ? std::string() : path.substr(0, p + 1);
}

}  // namespace

std::string format_timestamp(std::time_t t) {
    std::tm tm{};
    localtime_r(&t, &tm);
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%04d-%s-%02d %02d:%02d:%02d", tm.tm_year + 1900, kMonths[tm.tm_mon], tm.tm_mday,
                  tm.tm_hour, tm.tm_min, tm.tm_sec);
    return buf;
}

std::time_t parse_timestamp(const std::string &s) {
    int y = 0, d = 0, hh = 0, mm = 0, ss = 0, mon = -1;
    char month[16] = {0};
    if (std::sscanf(s.c_str(), "%d-%15[^-]-%d %d:%d:%d", &y, month, &d, &hh, &mm, &ss) != 6)
        init_error("Invalid timestamp '" + s + "'.");
    for (int i = 0; i < 12; ++i)
        if (strcasecmp(month, kMonths[i]) == 0) mon = i;
    if (mon < 0) {
        char *end = nullptr;
        long v = std::strtol(month, &end, 10);
        if (end && *end == '\0' && v >= 1 && v <= 12) mon = int(v) - 1;
    }
    if (mon < 0) init_error("Invalid timestamp '" + s + "'.");
    std::tm tm{};
    tm.tm_year = y - 1900;
    tm.tm_mon = mon;
    tm.tm_mday = d;
    tm.tm_hour = hh;
    tm.tm_min = mm;
    tm.tm_sec = ss;
    tm.tm_isdst = -1;
    return std::mktime(&tm);
}

std::string replace_extension(const std::string &path, const std::string &ext) {
    size_t slash = path.find_last_of('/');
    size_t dot = path.find_last_of('.');
    std::string stem = (dot != std::string::npos && (slash == std::string::npos || dot > slash) && dot != slash + 1)
                           ? path.substr(0, dot)
                           : path;
    return stem + "." + ext;
}

Fileset make_fileset(const std::string &task_path) {
    Fileset f;
    f.task = task_path;
    f.obs = replace_extension(task_path, "obs");
    f.data = replace_extension(task_path, "data");
    f.checkpoint = replace_extension(task_path, "checkpoint");
    f.ldf = replace_extension(task_path, "ldf");
    return f;
}

Task parse_task(const std::string &task_path, bool force_restart, bool touch_files) {
    Task t;
    t.files = make_fileset(task_path);
    if (!file_exists(task_path)) throw Error(ErrorType::IO, "Task file [" + task_path + "] does not exist.");
    t.doc = xml_parse_file(task_path);
    const XmlNode &doc = t.doc;

    validate(doc, "", {"task"}, {});
    validate(doc, "task", {"parameters"}, {}, {"measurements", "calculation"});
    validate(doc, "task.parameters", {"frequency", "cutoff", "lattice", "model"}, {});

    // computation status (src/TaskFileParser.cpp:31-73)
    const XmlNode *calc = at_path(doc, "task.calculation");
    const std::string *status = calc ? calc->attr("status") : nullptr;
    if (force_restart || !status) {
        t.status.status = CalcStatus::New;
    } else {
        auto need = [&](const char *key, const std::string &msg) -> std::time_t {
            const std::string *v = calc->attr(key);
            if (!v) init_error(msg);
            return parse_timestamp(*v);
        };
        if (*status == "running") {
            t.status.status = CalcStatus::Running;
            t.status.start_time = need("startTime", "Checkpoint is corrupted [start time is not specified].");
        } else if (*status == "postprocessing") {
            t.status.status = CalcStatus::Postprocessing;
            t.status.start_time = need("startTime", "Checkpoint is corrupted [start time is not specified].");
            t.status.checkpoint_time = need("checkpointTime", "Checkpoint is corrupted [checkpoint time is not specified].");
        } else if (*status == "finished") {
            t.status.status = CalcStatus::Finished;
            t.status.start_time = need("startTime", "Checkpoint is corrupted [start time is not specified].");
            t.status.checkpoint_time = need("checkpointTime", "Checkpoint is corrupted [checkpoint time is not specified].");
            t.status.end_time = need("endTime", "Cannot continue calculation of task. Checkpoint seems corrupted (end time is not specified).");
        } else {
            init_error("Checkpoint is corrupted [end time is not specified].");
        }
    }
    if (t.status.status == CalcStatus::New && touch_files) {
        for (const auto &f : {std::make_pair(std::string("Checkpoint"), t.files.checkpoint), std::make_pair(std::string("Data"), t.files.data)}) {
            if (!file_exists(f.second)) continue;
            if (!force_restart)
                throw Error(ErrorType::IO, f.first + " file [" + f.second + "] already exists. Specify the --forceRestart option to overwrite existing files.");
            std::remove(f.second.c_str());
        }
    }

    // frequency (src/TaskFileParser.cpp:103-148)
    validate(doc, "task.parameters.frequency", {}, {"discretization"}, {"min", "max", "count", "value"});
    const XmlNode &fnode = *at_path(doc, "task.parameters.frequency");
    const std::string fdisc = *fnode.attr("discretization");
    if (fdisc == "exponential") {
        validate(doc, "task.parameters.frequency", {"min", "max", "count"}, {"discretization"});
        float mn = to_float(text_of(doc, "task.parameters.frequency.min"));
        if (mn <= 0) init_error("Invalid task file. Parameter 'task.parameters.frequency.min' must be positive");
        float mx = to_float(text_of(doc, "task.parameters.frequency.max"));
        if (mx <= mn) init_error("Invalid task file. Parameter 'task.parameters.frequency.max' must be greater than 'task.parameters.frequency.min'");
        float count = to_float(text_of(doc, "task.parameters.frequency.count"));
        if (count <= 1) init_error("Invalid task file. Parameter 'task.parameters.frequency.count' must be greater than 2.");
        float step = powf(mx / mn, 1.0f / (count - 1));
        for (int i = 0; i < count; ++i) t.frequencies.push_back(mn * powf(step, float(i)));
    } else if (fdisc == "manual") {
        validate(doc, "task.parameters.frequency", {}, {"discretization"}, {"value"});
        for (const auto &c : fnode.children) {
            if (c.name != "value") continue;
            if (c.text.find_first_not_of(" \t\r\n") == std::string::npos)
                init_error("Invalid task file. Unspecified parameter value (task.parameters.frequency.value)");
            t.frequencies.push_back(to_float(c.text));
        }
        std::sort(t.frequencies.begin(), t.frequencies.end());
        for (size_t i = 0; i + 1 < t.frequencies.size(); ++i)
            if (t.frequencies[i] == t.frequencies[i + 1]) init_error("Invalid task file. Duplicate value in task.parameters.frequency.value");
    } else {
        init_error("Invalid task file. Unknown attribute value '" + fdisc + "' (task.parameters.frequency.discretization)");
    }
    if (t.frequencies.empty()) init_error("Invalid task file. No frequency values (task.parameters.frequency)");
    if (t.frequencies.front() <= 0) init_error("Invalid task file. Frequency values must be positive (task.parameters.frequency)");

    // cutoff (src/TaskFileParser.cpp:150-198)
    validate(doc, "task.parameters.cutoff", {}, {"discretization"}, {"min", "max", "step", "value"});
    const XmlNode &cnode = *at_path(doc, "task.parameters.cutoff");
    const std::string cdisc = *cnode.attr("discretization");
    if (cdisc == "exponential") {
        validate(doc, "task.parameters.cutoff", {"min", "max", "step"}, {"discretization"});
        float mn = to_float(text_of(doc, "task.parameters.cutoff.min"));
        if (mn <= 0) init_error("Invalid task file. Parameter 'task.parameters.cutoff.min' must be positive");
        float mx = to_float(text_of(doc, "task.parameters.cutoff.max"));
        if (mx <= mn) init_error("Invalid task file. Parameter 'task.parameters.cutoff.max' must be greater than 'task.parameters.cutoff.min'");
        float step = to_float(text_of(doc, "task.parameters.cutoff.step"));
        if (step <= 0 || step >= 1) init_error("Invalid task file. Parameter 'task.parameters.cutoff.step' must be in the range (0,1)");
        while (mx > mn) {
            t.cutoffs.push_back(mx);
            mx *= step;
        }
    } else if (cdisc == "manual") {
        validate(doc, "task.parameters.cutoff", {}, {"discretization"}, {"value"});
        for (const auto &c : cnode.children) {
            if (c.name != "value") continue;
            if (c.text.find_first_not_of(" \t\r\n") == std::string::npos)
                init_error("Invalid task file. Unspecified parameter value (task.parameters.cutoff.value)");
            t.cutoffs.push_back(to_float(c.text));
        }
        std::sort(t.cutoffs.begin(), t.cutoffs.end(), std::greater<float>());
    } else {
        init_error("Invalid task file. Unknown attribute value '" + cdisc + "' (task.parameters.cutoff.discretization)");
    }
    if (t.cutoffs.empty()) init_error("Invalid task file. No cutoff values (task.parameters.cutoff)");

    // lattice and model (src/TaskFileParser.cpp:200-229)
    validate(doc, "task.parameters.lattice", {}, {"name", "range"});
    const XmlNode &mnode = *at_path(doc, "task.parameters.model");
    for (const char *a : {"name", "symmetry"})
        if (!mnode.attr(a)) init_error(std::string("Invalid task file. Missing attribute 'task.parameters.model.") + a + "'.");
    const XmlNode &lnode = *at_path(doc, "task.parameters.lattice");
    try {
        t.range = std::stoi(*lnode.attr("range"));
    } catch (const std::exception &) {
        init_error("Invalid task file. Parameter 'task.parameters.lattice.range' is not an integer");
    }
    t.lattice = *lnode.attr("name");
    t.model = *mnode.attr("name");
    t.symmetry = *mnode.attr("symmetry");
    for (const auto &c : mnode.children) {
        if (c.text.find_first_not_of(" \t\r\n") == std::string::npos)
            init_error("Invalid task file. Unspecified parameter value (task.parameters.model." + c.name + ")");
        if (!t.model_options.emplace(c.name, c.text).second)
            init_error("Invalid task file. Multiple definitions of parameter 'task.parameters.model." + c.name + "'");
    }

    // measurements (src/TaskFileParser.cpp:231-306)
    if (at_path(doc, "task.measurements")) {
        validate(doc, "task.measurements", {}, {}, {"measurement"});
        for (const auto &m : at_path(doc, "task.measurements")->children) {
            if (m.name != "measurement") continue;
            const std::string where = "task.measurements.measurement";
            if (!m.attr("name")) init_error("Invalid task file. Missing attribute '" + where + ".name'.");
            for (const auto &a : m.attrs) {
                static const std::set<std::string> ok = {"name", "output", "method", "minCutoff", "maxCutoff"};
                if (!ok.count(a.first)) init_error("Invalid task file. Unknown attribute '" + where + "." + a.first + "'.");
            }
            MeasurementSpec s;
            s.name = *m.attr("name");
            s.output = m.attr("output") ? directory_of(task_path) + *m.attr("output") : t.files.obs;
            if (t.status.status == CalcStatus::New && touch_files && file_exists(s.output)) {
                if (!force_restart)
                    throw Error(ErrorType::IO, "Observable file [" + s.output + "] already exists. Specify the --forceRestart option to overwrite existing files.");
                std::remove(s.output.c_str());
            }
            s.defer = m.attr("method") && *m.attr("method") == "defer";
            if (m.attr("minCutoff")) s.min_cutoff = to_float(*m.attr("minCutoff"));
            if (m.attr("maxCutoff")) s.max_cutoff = to_float(*m.attr("maxCutoff"));
            for (const auto &c : m.children) {
                if (c.text.find_first_not_of(" \t\r\n") == std::string::npos)
                    init_error("Invalid task file. Unspecified parameter value (" + where + "." + c.name + ")");
                s.options.emplace_back(c.name, c.text);
            }
            t.measurements.push_back(s);
        }
    }
    return t;
}

void write_task(Task &task, const ComputationStatus &st) {
    XmlNode *root = nullptr;
    for (auto &c : task.doc.children)
        if (c.name == "task") root = &c;
    if (!root) throw Error(ErrorType::Internal, "task document has no <task> element");
    root->children.erase(std::remove_if(root->children.begin(), root->children.end(),
                                        [](const XmlNode &n) { return n.name == "calculation"; }),
                         root->children.end());
    if (st.status != CalcStatus::New) {
        XmlNode calc;
        calc.name = "calculation";
        calc.attrs.emplace_back("startTime", format_timestamp(st.start_time));
        calc.attrs.emplace_back("checkpointTime", format_timestamp(st.checkpoint_time));
        if (st.status == CalcStatus::Running) {
            calc.attrs.emplace_back("status", "running");
        } else if (st.status == CalcStatus::Postprocessing) {
            calc.attrs.emplace_back("status", "postprocessing");
        } else {
            calc.attrs.emplace_back("endTime", format_timestamp(st.end_time));
            calc.attrs.emplace_back("status", "finished");
        }
        root->children.push_back(calc);
    }
    task.status = st;
    std::string out = xml_serialize(task.doc);
    std::ofstream f(task.files.task, std::ios::out | std::ios::trunc);
    if (!f.is_open()) throw Error(ErrorType::IO, "Could not open task file for writing");
    f << out;
    if (!f.good()) throw Error(ErrorType::IO, "Could not write task file");
}

}  // namespace spn
