// hpss_host.cpp -- implementation of the host side declared in hpss_host.hpp.
#include "hpss_host.hpp"

#include <algorithm>
#include <cerrno>
#include <cmath>
#include <cstring>
#include <ctime>
#include <filesystem>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <limits>
#include <numeric>
#include <sstream>
#include <thread>

namespace hpsshost {

// ================================================================ logging
Logger *Logger::getInstance() {
    static Logger instance;
    return &instance;
}

void Logger::print(LogLevel lvl, const std::string &message) {
    static const char *names[] = {"ERROR", "INFO", "LOW", "HIGH", "DEBUG"};
    std::ostream &os = lvl == LogLevel::ERROR ? std::cerr : std::cout;
    os << "[" << names[(int)lvl] << "] " << message << std::endl;
}

// ================================================================ model
namespace Utils {
// Utils::midpoint_axis / halfoffset_axis / midpoint / halfoffset
// (common/src/model/Utils.cpp:8-52): float arithmetic in the same order.
static float fscalco(const trace_info_t &t) {
    float scalco = static_cast<float>(t.scalco);
    return t.scalco >= 0 ? scalco : -1.0f / scalco;
}
float midpoint(const trace_info_t &t, float az) {
    float fs = fscalco(t);
    float mx = fs * static_cast<float>(t.gx + t.sx) * 0.5f;
    float my = fs * static_cast<float>(t.gy + t.sy) * 0.5f;
    return mx * std::sin(az) + my * std::cos(az);
}
float halfoffset(const trace_info_t &t, float az) {
    float fs = fscalco(t);
    float hx = fs * static_cast<float>(t.gx - t.sx) * 0.5f;
    float hy = fs * static_cast<float>(t.gy - t.sy) * 0.5f;
    return hx * std::sin(az) + hy * std::cos(az);
}
float degreesToRad(float degree) { return degree * static_cast<float>(M_PI) / 180.0f; }
}  // namespace Utils

Trace::Trace() { std::memset(&info, 0, sizeof(info)); }

// Trace::read (common/src/model/Trace.cpp:45-61): a header read that hits the
// end of the file leaves the trace empty; a truncated sample block throws.
bool Trace::read(std::ifstream &fin, float az) {
    if (fin.read(reinterpret_cast<char *>(&info), sizeof(trace_info_t)).eof()) {
        std::memset(&info, 0, sizeof(info));
        return false;
    }
    midpoint = Utils::midpoint(info, az);
    halfoffset = Utils::halfoffset(info, az);
    samples.resize(info.ns);
    if (fin.read(reinterpret_cast<char *>(samples.data()), samples.size() * sizeof(float)).eof())
        throw std::runtime_error("end of file reached before reading all samples.");
    return true;
}

bool Trace::operator<(const Trace &o) const {
    if (midpoint < o.midpoint) return true;
    return midpoint == o.midpoint && halfoffset < o.halfoffset;
}

Gather::Gather()
    : lowestAllowedMidpoint(std::numeric_limits<float>::min()),
      biggestAllowedMidpoint(std::numeric_limits<float>::max()) {}

Gather *Gather::getInstance() {
    static Gather instance;
    return &instance;
}

void Gather::reset() {
    cdps.clear();
    traces.clear();
    samplesPerTrace = 0;
    samplesCount = 0;
}

void Gather::setAzimuthInDegree(float deg) {
    azimuthInDegrees = deg;
    azimuthInRad = Utils::degreesToRad(deg);
}

// readGatherFromFile (Gather.cpp:49-126), including its `while (!eof)` loop
// that runs once more after the last trace and inserts a CDP at midpoint 0.
void Gather::readGatherFromFile(const std::string &inFile) {
    std::ifstream fin(inFile, std::ios::binary);
    if (!fin.is_open()) throw std::invalid_argument(inFile + " couldn't be read.");
    samplesCount = 0;
    while (!fin.eof()) {
        Trace trace;
        trace.read(fin, azimuthInRad);
        float m = trace.getMidpoint(), h = trace.getHalfoffset();
        if (!samplesPerTrace) {
            samplesPerTrace = trace.getSampleCount();
            dt = trace.getInfo().dt;
            dtInSeconds = static_cast<float>(dt) * 1e-6f;
            tauIndexDisplacement = dtInSeconds > 0 ? static_cast<int>(tau / dtInSeconds) : 0;
            windowSize = 2 * tauIndexDisplacement + 1;
        }
        if (cdps.find(m) == cdps.end()) {
            trace_info_t ci = trace.getInfo();
            ci.offset = 0;
            ci.sx = ci.gx = (trace.getInfo().sx + trace.getInfo().gx) >> 1;
            ci.sy = ci.gy = (trace.getInfo().sy + trace.getInfo().gy) >> 1;
            LOGH("CDP not found. Creating a new one with midpoint = " << m);
            cdps[m] = Cdp(m, ci);
        }
        if (samplesPerTrace != trace.getSampleCount()) continue;
        if (std::fabs(h) > aph) continue;
        if (!trace.isMidpointInRange(lowestAllowedMidpoint, biggestAllowedMidpoint)) continue;
        samplesCount += trace.getSampleCount();
        cdps[m].incrementTraceCountBy(1);
        cdps[m].incrementSampleCountBy(trace.getSampleCount());
        traces.push_back(std::move(trace));
    }
    // equal (m, h) keys keep file order (the reference's std::sort leaves them unspecified)
    std::stable_sort(traces.begin(), traces.end());
    LOGI("Number of CDPs = " << cdps.size());
    LOGI("Number of traces in the gather = " << traces.size());
    LOGI("Number of samples per trace = " << samplesPerTrace);
}

const std::string Gather::toString() const {
    std::ostringstream s;
    s << "Samples per trace = " << samplesPerTrace << std::endl;
    s << "Total traces count = " << traces.size() << std::endl;
    s << "Total samples = " << samplesCount << std::endl;
    s << "CDPs = " << cdps.size() << std::endl;
    s << "apm = " << apm << " m" << std::endl;
    s << "aph = " << aph << " m" << std::endl;
    s << "tau = " << tau << std::endl;
    s << "azimuth = " << azimuthInRad << " rad" << std::endl;
    return s.str();
}

// ================================================================ traveltime
std::string Traveltime::getDescriptionForResult(unsigned i) const {
    if (i == 0) return "coherence";
    if (i == 1) return "stack";
    return params[i - 2].getParameterDescription();
}

std::string Traveltime::toString() const {
    std::ostringstream s;
    s << "Name = " << getTraveltimeWord() << std::endl;
    s << "h0 = " << getReferenceHalfoffset() << std::endl;
    for (unsigned i = 0; i < getNumberOfParameters(); i++)
        s << getDescriptionForParameter(i) << " in [" << getLowerBoundForParameter(i) << ", "
          << getUpperBoundForParameter(i) << "]";
    return s.str();
}

std::string CommonReflectionSurface::toString() const {
    std::ostringstream s;
    s << Traveltime::toString() << std::endl;
    s << "v0 = " << v0 << std::endl << "ain = " << Utils::degreesToRad(ainDeg) << " rad" << std::endl;
    s << "bpctg = " << bpctg << std::endl;
    return s.str();
}

std::string StretchFreeTraveltimeWrapper::getDescriptionForResult(unsigned i) const {
    if (i == 0) return "coherence";
    if (i == 1) return "stack";
    return "n";
}

namespace TraveltimeBuilder {
static void setBounds(Traveltime *t, const std::vector<float> &lo, const std::vector<float> &hi,
                      const char *name) {
    unsigned n = t->getNumberOfParameters();
    if (lo.size() != n || hi.size() != n) {
        std::ostringstream e;
        e << name << " requires exact " << n << " lower and upper bounds.";
        delete t;
        throw std::logic_error(e.str());
    }
    for (unsigned i = 0; i < n; i++) {
        t->updateLowerBoundForParameter(i, lo[i]);
        t->updateUpperBoundForParameter(i, hi[i]);
    }
}
Traveltime *buildCommonMidPoint(const std::vector<float> &lo, const std::vector<float> &hi) {
    Traveltime *t = new CommonMidPoint();
    setBounds(t, lo, hi, "CMP");
    return t;
}
// A and B bounds are derived (TraveltimeBuilder.cpp:45-76).
Traveltime *buildZeroOffsetCommonReflectionSurface(const std::vector<float> &lo,
                                                   const std::vector<float> &hi, float v0,
                                                   float aIn, float bPctg) {
    if (lo.empty() || hi.empty())
        throw std::logic_error("ZOCRS requires at least a single lower/upper bound.");
    auto *t = new CommonReflectionSurface();
    t->updateLowerBoundForParameter(0, lo[0]);
    t->updateUpperBoundForParameter(0, hi[0]);
    t->v0 = v0;
    t->ainDeg = aIn;
    t->bpctg = bPctg;
    float minV = lo[0];
    float aMax = 2.0f * std::sin(Utils::degreesToRad(aIn)) / v0;
    float bMax = bPctg * 4 / (minV * minV);
    t->updateLowerBoundForParameter(1, -aMax);
    t->updateUpperBoundForParameter(1, aMax);
    t->updateLowerBoundForParameter(2, -bMax);
    t->updateUpperBoundForParameter(2, bMax);
    return t;
}
Traveltime *buildOffsetContinuationTrajectory(const std::vector<float> &lo,
                                              const std::vector<float> &hi, float h0) {
    Traveltime *t = new OffsetContinuationTrajectory();
    setBounds(t, lo, hi, "OCT");
    t->updateReferenceHalfoffset(h0);
    return t;
}
}  // namespace TraveltimeBuilder

// ================================================================ results
const std::string &statisticName(StatisticResult r) {
    static const std::string names[] = {"efficiency", "interpolations_per_sec",
                                        "selected_traces", "total_selection_kernel_exec_time",
                                        "total_kernel_exec_time"};
    return names[(int)r];
}

const std::vector<float> &MidpointResult::get(float m0) const {
    auto it = results.find(m0);
    if (it == results.end()) throw std::invalid_argument("Empty result for given midpoint.");
    return it->second;
}

float StatisticalMidpointResult::getStatisticalResultForMidpoint(float m0) const {
    auto it = stats.find(m0);
    if (it == stats.end()) throw std::invalid_argument("Empty result for given midpoint.");
    return it->second;
}

// StatisticalMidpointResult::getAverageOfAllMidpoints: zeros are left out of
// the sum but not of the count (StatisticalMidpointResult.cpp).
float StatisticalMidpointResult::getAverageOfAllMidpoints() const {
    if (stats.empty()) return 0;
    float sum = 0;
    for (auto &kv : stats)
        if (kv.second != 0) sum += kv.second;
    return sum / static_cast<float>(stats.size());
}

void ResultSet::setAllResultsForMidpoint(float m0, const std::vector<float> &array,
                                         size_t offset) {
    for (size_t i = 0; i < resultArray.size(); i++) {
        auto b = array.cbegin() + offset + i * samplesPerResult;
        resultArray[i].save(m0, b, b + samplesPerResult);
    }
}

const StatisticalMidpointResult &ResultSet::get(StatisticResult s) const {
    auto it = stats.find(s);
    if (it == stats.end()) throw std::invalid_argument("Empty result for statistical result.");
    return it->second;
}

// ================================================================ devices + algorithms
void check(hpss_handle h, hpss_status rc) {
    if (rc == HPSS_OK) return;
    std::string msg = hpss_last_error(h);
    if (rc == HPSS_ERR_INVALID_ARGUMENT) throw std::invalid_argument(msg);
    if (rc == HPSS_ERR_LOGIC) throw std::logic_error(msg);
    throw std::runtime_error(msg);
}

DeviceContext::DeviceContext(unsigned devId) : deviceId(devId) {
    check(nullptr, hpss_create((int)devId, &h));
}

DeviceContext::~DeviceContext() { hpss_destroy(h); }

ComputeAlgorithm::ComputeAlgorithm(const std::string &name, std::shared_ptr<Traveltime> model,
                                   std::shared_ptr<DeviceContext> ctx, unsigned tc)
    : algorithmName(name), deviceContext(std::move(ctx)), traveltime(std::move(model)),
      threadCount(tc) {}

float ComputeAlgorithm::getStatisticalResult(StatisticResult r) const {
    auto it = computedStatisticalResults.find((int)r);
    if (it == computedStatisticalResults.end())
        throw std::invalid_argument("Couldn't find value for statistical result.");
    return it->second;
}

// Upload the line and set model and window (copyGatherDataToDevice and the
// parameter set-up of the reference's setUp methods).
void ComputeAlgorithm::setUp() {
    Gather *g = Gather::getInstance();
    hpss_handle h = deviceContext->handle();
    const unsigned n = g->getTotalTracesCount(), S = g->getSamplesPerTrace();
    std::vector<float> smp((size_t)n * S), m(n), hoff(n);
    for (unsigned i = 0; i < n; i++) {
        const Trace &t = g->getTraceAtIndex(i);
        std::copy(t.getSamples().begin(), t.getSamples().end(), smp.begin() + (size_t)i * S);
        m[i] = t.getMidpoint();
        hoff[i] = t.getHalfoffset();
    }
    check(h, hpss_upload_gather(h, smp.data(), m.data(), hoff.data(), n, S ? S : 1,
                                g->getSamplePeriodInSeconds() > 0 ? g->getSamplePeriodInSeconds()
                                                                  : 1e-3f,
                                storage));
    check(h, hpss_set_grid_mode(h, gridMode));
    check(h, hpss_set_precision(h, precisionFlags));
    const unsigned np = traveltime->getNumberOfParameters();
    std::vector<float> lo(np), hi(np);
    for (unsigned j = 0; j < np; j++) {
        lo[j] = traveltime->getLowerBoundForParameter(j);
        hi[j] = traveltime->getUpperBoundForParameter(j);
    }
    check(h, hpss_set_traveltime(h, traveltime->getModel(), np, lo.data(), hi.data(),
                                 g->getApm(), traveltime->getReferenceHalfoffset()));
    check(h, hpss_set_window(h, g->getTauIndexDisplacement()));
    computedResults.assign((size_t)resultRows() * S, 0.f);
    isSet = true;
}

void ComputeAlgorithm::computeSemblanceAndParametersForMidpoint(float m0) {
    std::vector<float> res;
    std::vector<std::map<StatisticResult, float>> st;
    computeSemblanceAndParametersForMidpoints({m0}, res, st);
    computedResults = res;
    for (auto &kv : st[0]) computedStatisticalResults[(int)kv.first] = kv.second;
}

// Per-midpoint statistics of a batched call (StatisticResult semantics,
// ComputeAlgorithm.cpp:71-105): kernel time is shared out by each midpoint's
// share of the evaluations.
void ComputeAlgorithm::fillStats(const std::vector<float> &m0s, const hpss_stats &st,
                                 double perCandidateFactor,
                                 std::vector<std::map<StatisticResult, float>> &stats) {
    hpss_handle h = deviceContext->handle();
    std::vector<uint32_t> counts(m0s.size(), 0);
    if (traveltime->getModel() != OCT || algorithmName == "linear-search")
        check(h, hpss_select_traces(h, m0s.data(), (uint32_t)m0s.size(), counts.data()));
    const double total = std::max(st.evals, 1.0);
    const unsigned w = Gather::getInstance()->getWindowSize();
    const double rate = st.kernel_ms > 0 ? w * (st.evals - st.not_used) / (st.kernel_ms / 1e3) : 0;
    const double eff = st.evals > 0 ? 1.0 - st.not_used / st.evals : 1.0;
    stats.assign(m0s.size(), {});
    for (size_t i = 0; i < m0s.size(); i++) {
        double share = counts[i] * perCandidateFactor / total;
        auto &s = stats[i];
        s[StatisticResult::EFFICIENCY] = (float)eff;
        s[StatisticResult::INTR_PER_SEC] = (float)rate;
        s[StatisticResult::SELECTED_TRACES] = (float)counts[i];
        s[StatisticResult::TOTAL_SELECTION_KERNEL_EXECUTION_TIME] =
            (float)(st.selection_ms / 1e3 / std::max<size_t>(m0s.size(), 1));
        s[StatisticResult::TOTAL_KERNEL_EXECUTION_TIME] = (float)(st.kernel_ms / 1e3 * share);
    }
}

LinearSearchAlgorithm::LinearSearchAlgorithm(std::shared_ptr<Traveltime> model,
                                             std::shared_ptr<DeviceContext> ctx, unsigned tc,
                                             const std::vector<int> &g, int k)
    : ComputeAlgorithm("linear-search", std::move(model), std::move(ctx), tc), kernel(k) {
    for (int v : g) granularity.push_back((uint32_t)v);
}

unsigned LinearSearchAlgorithm::getTotalNumberOfParameters() const {
    return std::accumulate(granularity.begin(), granularity.end(), 1u, std::multiplies<unsigned>());
}

void LinearSearchAlgorithm::computeSemblanceAndParametersForMidpoints(
    const std::vector<float> &m0s, std::vector<float> &results,
    std::vector<std::map<StatisticResult, float>> &stats) {
    hpss_handle h = deviceContext->handle();
    const unsigned S = Gather::getInstance()->getSamplesPerTrace();
    results.assign(m0s.size() * resultRows() * S, 0.f);
    hpss_stats st{};
    check(h, hpss_linear_search(h, m0s.data(), (uint32_t)m0s.size(), granularity.data(), kernel,
                                results.data(), &st));
    fillStats(m0s, st, (double)S * getTotalNumberOfParameters(), stats);
}

std::string LinearSearchAlgorithm::toString() const {
    std::ostringstream s;
    s << "Total number of parameters = " << getTotalNumberOfParameters() << std::endl;
    for (unsigned i = 0; i < traveltime->getNumberOfParameters(); i++)
        s << "# of discrete values for " << traveltime->getDescriptionForParameter(i) << " = "
          << granularity[i] << std::endl;
    s << "Thread count = " << threadCount << std::endl;
    return s.str();
}

DifferentialEvolutionAlgorithm::DifferentialEvolutionAlgorithm(
    std::shared_ptr<Traveltime> model, std::shared_ptr<DeviceContext> ctx, unsigned tc,
    unsigned gen, unsigned pop, float f, float cr, uint64_t sd)
    : ComputeAlgorithm("de", std::move(model), std::move(ctx), tc), generations(gen),
      individualsPerPopulation(pop), F(f), CR(cr), seed(sd) {}

void DifferentialEvolutionAlgorithm::computeSemblanceAndParametersForMidpoints(
    const std::vector<float> &m0s, std::vector<float> &results,
    std::vector<std::map<StatisticResult, float>> &stats) {
    hpss_handle h = deviceContext->handle();
    const unsigned S = Gather::getInstance()->getSamplesPerTrace();
    results.assign(m0s.size() * resultRows() * S, 0.f);
    hpss_stats st{};
    check(h, hpss_differential_evolution(h, m0s.data(), (uint32_t)m0s.size(),
                                         individualsPerPopulation, generations, F, CR, seed,
                                         results.data(), &st));
    fillStats(m0s, st, (double)S * individualsPerPopulation * generations, stats);
}

std::string DifferentialEvolutionAlgorithm::toString() const {
    std::ostringstream s;
    s << "Total number of generations = " << generations << std::endl;
    s << "Total number of ind. per population = " << individualsPerPopulation << std::endl;
    s << "F = " << F << ", CR = " << CR << ", seed = " << seed << std::endl;
    return s.str();
}

StretchFreeAlgorithm::StretchFreeAlgorithm(std::shared_ptr<Traveltime> model,
                                           std::shared_ptr<DeviceContext> ctx, unsigned tc,
                                           const std::vector<std::string> &files)
    : ComputeAlgorithm("strecth-free", std::move(model), std::move(ctx), tc),
      parameterFileArray(files) {}

// readNonStretchedFreeParameterFromFile (StretchFreeAlgorithm.cpp:101-125):
// one trace per parameter file per CDP, in CDP-map order.
void StretchFreeAlgorithm::setUp() {
    ComputeAlgorithm::setUp();
    Gather *g = Gather::getInstance();
    const unsigned np = traveltime->getNumberOfParameters(), S = g->getSamplesPerTrace();
    std::vector<std::ifstream> files(np);
    for (unsigned i = 0; i < np; i++) {
        files[i].open(parameterFileArray[i], std::ios::binary);
        if (!files[i].is_open())
            throw std::invalid_argument(parameterFileArray[i] + " couldn't be read.");
    }
    for (auto &kv : g->getCdps()) {
        std::vector<float> p((size_t)np * S, 0.f);
        for (unsigned i = 0; i < np; i++) {
            Trace t;
            t.read(files[i], g->getAzimuthInRad());
            const auto &smp = t.getSamples();
            std::copy(smp.begin(), smp.begin() + std::min<size_t>(smp.size(), S),
                      p.begin() + (size_t)i * S);
        }
        nonStretchFreeParameters[kv.first] = std::move(p);
    }
}

void StretchFreeAlgorithm::computeSemblanceAndParametersForMidpoints(
    const std::vector<float> &m0s, std::vector<float> &results,
    std::vector<std::map<StatisticResult, float>> &stats) {
    hpss_handle h = deviceContext->handle();
    const unsigned S = Gather::getInstance()->getSamplesPerTrace();
    const unsigned np = traveltime->getNumberOfParameters();
    std::vector<float> prior;
    prior.reserve(m0s.size() * np * S);
    for (float m0 : m0s) {
        auto it = nonStretchFreeParameters.find(m0);
        if (it == nonStretchFreeParameters.end())
            prior.insert(prior.end(), (size_t)np * S, 0.f);
        else
            prior.insert(prior.end(), it->second.begin(), it->second.end());
    }
    results.assign(m0s.size() * 3 * S, 0.f);
    hpss_stats st{};
    check(h, hpss_stretch_free(h, m0s.data(), (uint32_t)m0s.size(), prior.data(), NMAX,
                               results.data(), &st));
    fillStats(m0s, st, (double)S * (2 * NMAX + 1), stats);
}

std::string StretchFreeAlgorithm::toString() const {
    std::ostringstream s;
    s << "Total number of parameters = " << 2 * NMAX + 1 << std::endl;
    s << "N in [ " << -NMAX << "," << NMAX << "]" << std::endl;
    s << "Parameter files: " << std::endl;
    for (auto &f : parameterFileArray) s << f << std::endl;
    return s.str();
}

// CudaComputeAlgorithmBuilder's checks (CudaComputeAlgorithmBuilder.cu:20-72).
LinearSearchAlgorithm *Gb300ComputeAlgorithmBuilder::buildLinearSearchAlgorithm(
    std::shared_ptr<Traveltime> tt, std::shared_ptr<DeviceContext> ctx, unsigned threadCount,
    const std::vector<int> &g) {
    if (g.size() != tt->getNumberOfParameters()) {
        std::ostringstream e;
        e << tt->getTraveltimeWord() << " requires exact " << tt->getNumberOfParameters()
          << " discretization granularities.";
        throw std::logic_error(e.str());
    }
    auto *alg = new LinearSearchAlgorithm(tt, ctx, threadCount, g, opts.kernel);
    alg->setEngineStorage(opts.storage);
    alg->setEngineGridMode(opts.gridMode);
    alg->setEnginePrecision(opts.precisionFlags);
    return alg;
}

DifferentialEvolutionAlgorithm *Gb300ComputeAlgorithmBuilder::buildDifferentialEvolutionAlgorithm(
    std::shared_ptr<Traveltime> tt, std::shared_ptr<DeviceContext> ctx, unsigned threadCount,
    unsigned generations, unsigned population) {
    uint64_t seed = opts.seedGiven ? opts.seed : (uint64_t)time(nullptr);
    auto *alg = new DifferentialEvolutionAlgorithm(tt, ctx, threadCount, generations, population,
                                                   opts.deF, opts.deCR, seed);
    alg->setEngineStorage(opts.storage);
    return alg;
}

StretchFreeAlgorithm *Gb300ComputeAlgorithmBuilder::buildStretchFreeAlgorithm(
    std::shared_ptr<Traveltime> tt, std::shared_ptr<DeviceContext> ctx, unsigned threadCount,
    const std::vector<std::string> &files) {
    if (files.size() != tt->getNumberOfParameters()) {
        std::ostringstream e;
        e << tt->getTraveltimeWord() << " requires exact " << tt->getNumberOfParameters()
          << " parameter files.";
        throw std::logic_error(e.str());
    }
    return new StretchFreeAlgorithm(tt, ctx, threadCount, files);
}

// ================================================================ output
Dumper::Dumper(const std::string &path, const std::string &dataFile, const std::string &method,
               const std::string &traveltime) {
    std::ostringstream s;
    time_t t = time(nullptr);
    tm *now = localtime(&t);
    s << path << "/" << dataFile << "_" << method << "_" << traveltime << "_"
      << std::put_time(now, "%Y%m%d_%H%M") << "/";
    outputDirectoryPath = s.str();
}

void Dumper::createDir() const {
    if (std::filesystem::exists(outputDirectoryPath)) return;
    if (!std::filesystem::create_directory(outputDirectoryPath))
        throw std::runtime_error("Directory couldn't be created");
}

void Dumper::dumpGatherParameters(const std::string &file) const {
    std::ofstream o(outputDirectoryPath + "gather.txt");
    if (!o.is_open()) throw std::runtime_error("Couldn't open file gather.txt");
    o << "==== Gather Summary ====" << std::endl;
    o << "Input file = " << file << std::endl;
    o << Gather::getInstance()->toString() << std::endl;
}

void Dumper::dumpTraveltime(const Traveltime *t) const {
    std::ofstream o(outputDirectoryPath + "traveltime.txt");
    if (!o.is_open()) throw std::runtime_error("Couldn't open traveltime.txt");
    o << "==== Model Summary ====" << std::endl << t->toString() << std::endl;
}

void Dumper::dumpAlgorithm(const ComputeAlgorithm *a) const {
    std::ofstream o(outputDirectoryPath + "algorithm.txt");
    if (!o.is_open()) throw std::runtime_error("Couldn't open algorithm.txt");
    o << "==== Compute Algorithm Summary ====" << std::endl << a->toString() << std::endl;
}

// Dumper::dumpResult (Dumper.cpp:77-114): one trace per CDP in map order,
// header = the CDP's header.
void Dumper::dumpResult(const std::string &name, const MidpointResult &r) const {
    std::ofstream o(outputDirectoryPath + name + ".su", std::ios::binary);
    if (!o.is_open()) throw std::runtime_error("Couldn't open " + name + ".su");
    for (auto &kv : Gather::getInstance()->getCdps()) {
        const std::vector<float> &samples = r.get(kv.first);
        trace_info_t info = kv.second.getCdpInfo();
        info.ns = (uint16_t)samples.size();
        o.write(reinterpret_cast<const char *>(&info), sizeof(info));
        o.write(reinterpret_cast<const char *>(samples.data()), samples.size() * sizeof(float));
    }
}

void Dumper::dumpStatisticalResult(const std::string &name,
                                   const StatisticalMidpointResult &r) const {
    std::ofstream o(outputDirectoryPath + name + ".csv");
    if (!o.is_open()) throw std::runtime_error("Couldn't open " + name + ".csv");
    for (auto &kv : Gather::getInstance()->getCdps())
        o << kv.first << "," << r.getStatisticalResultForMidpoint(kv.first) << std::endl;
}

// ================================================================ cli
Parser::Parser() {
    // the reference's flag table (common/src/parser/Parser.cpp:13-35)
    add("aph", "APH constant.", true);
    add("apm", "APM constant.", true);
    add("ain", "Angle in degrees to be used during computation of A for ZO-CRS.");
    add("azimuth", "Azimuth angle in degrees.", true);
    add("bpctg", "Percentage of C that will be used to compute B for ZO-CRS.");
    add("h0", "h0 constant.");
    add("help", "Produce help message.", false, false, "", true);
    add("highest-midpoint", "Higher bound value for a CDP midpoint.");
    add("input", "*.su input data file.", true);
    add("lower-bounds", "Lower bound for traveltime parameters.", true, true);
    add("lowest-midpoint", "Lower bound value for a CDP midpoint.");
    add("kernel-path", "OpenCL's kernel location (accepted, unused).");
    add("output", "*.su output data prefix.", true);
    add("tau", "Semblance processing window given by w = 2 * tau + 1.");
    add("thread-count", "GPU thread count (accepted; the engine sizes its own launches).", false,
        false, "64");
    add("traveltime", "Traveltime traveltime to be used.", true);
    add("upper-bounds", "Upper bounds for traveltime parameters.", true, true);
    add("v0", "Velocity used to compute ZO-CRS A parameter.");
    add("verbose", "Verbosity level. Must be in the [0..4] integer range.");
    // engine options (no reference counterpart)
    add("kernel", "Engine kernel: tuned (default), tuned-exact or plain.", false, false, "tuned");
    add("precision", "Amplitude storage on the device: fp32 (default), bf16 or fp16.", false,
        false, "fp32");
    add("fp64-traveltime", "Linear search: ZO-CRS / OCT traveltime in FP64 (plain kernel).",
        false, false, "", true);
    add("compensated-sums", "Linear search: compensated window sums above 4096 terms "
        "(plain kernel).", false, false, "", true);
    add("grid-mode", "Linear-search grid: reference (default; uniform in v, upper bound "
        "excluded) or inclusive (both bounds, velocity uniform in 4/v^2).", false, false,
        "reference");
}

void Parser::add(const std::string &name, const std::string &help, bool required, bool multi,
                 const std::string &def, bool flag) {
    Option o;
    o.name = name;
    o.help = help;
    o.required = required;
    o.multi = multi;
    o.def = def;
    o.flag = flag;
    options.push_back(o);
}

// Long options only ("--name value", "--name=value"); multi-token options
// take every following token until the next "--" option.
void Parser::parseArguments(int argc, const char *argv[]) {
    try {
        values.clear();
        for (int i = 1; i < argc; i++) {
            std::string a = argv[i];
            if (a.rfind("--", 0) != 0)
                throw std::invalid_argument("unexpected positional argument '" + a + "'");
            std::string name = a.substr(2), inlineVal;
            bool hasInline = false;
            auto eq = name.find('=');
            if (eq != std::string::npos) {
                inlineVal = name.substr(eq + 1);
                name = name.substr(0, eq);
                hasInline = true;
            }
            auto it = std::find_if(options.begin(), options.end(),
                                   [&](const Option &o) { return o.name == name; });
            if (it == options.end())
                throw std::invalid_argument("unrecognised option '--" + name + "'");
            auto &v = values[name];
            if (it->flag) {
                v.push_back("1");
                continue;
            }
            if (hasInline) {
                v.push_back(inlineVal);
                continue;
            }
            int taken = 0;
            while (i + 1 < argc && std::string(argv[i + 1]).rfind("--", 0) != 0) {
                v.push_back(argv[++i]);
                taken++;
                if (!it->multi) break;
            }
            if (taken == 0)
                throw std::invalid_argument("the required argument for option '--" + name +
                                            "' is missing");
        }
        for (auto &o : options) {
            if (o.required && !values.count(o.name))
                throw std::invalid_argument("the option '--" + o.name + "' is required but missing");
            if (!o.def.empty() && !values.count(o.name)) values[o.name] = {o.def};
        }
        if (has("verbose"))
            Logger::getInstance()->setVerbosity(static_cast<LogLevel>(std::min(u("verbose"), 4u)));
    } catch (const std::invalid_argument &e) {
        throw std::invalid_argument(std::string("Unable to parse input arguments: ") + e.what());
    }
}

std::string Parser::str(const std::string &n) const {
    auto it = values.find(n);
    if (it == values.end() || it->second.empty())
        throw std::invalid_argument("option '--" + n + "' not provided");
    return it->second.front();
}
float Parser::f(const std::string &n) const { return std::stof(str(n)); }
unsigned Parser::u(const std::string &n) const { return (unsigned)std::stoul(str(n)); }
std::vector<float> Parser::floats(const std::string &n) const {
    std::vector<float> r;
    auto it = values.find(n);
    if (it != values.end())
        for (auto &s : it->second) r.push_back(std::stof(s));
    return r;
}
std::vector<int> Parser::ints(const std::string &n) const {
    std::vector<int> r;
    auto it = values.find(n);
    if (it != values.end())
        for (auto &s : it->second) r.push_back(std::stoi(s));
    return r;
}

std::string Parser::getFilename() const {
    return std::filesystem::path(getInputFilePath()).stem().string();
}
std::string Parser::getInputFilePath() const {
    if (has("input")) return str("input");
    throw std::invalid_argument("Input data file not provided.");
}
std::string Parser::getOutputDirectory() const {
    if (has("output")) return str("output");
    throw std::invalid_argument("Output path not provided.");
}
unsigned Parser::getGpuThreadCount() const { return u("thread-count"); }

EngineOptions Parser::engineOptions() const {
    EngineOptions o;
    if (has("kernel")) {
        std::string k = str("kernel");
        if (k == "plain") o.kernel = HPSS_KERNEL_PLAIN;
        else if (k == "tuned") o.kernel = HPSS_KERNEL_TUNED;
        else if (k == "tuned-exact") o.kernel = HPSS_KERNEL_TUNED_EXACT;
        else throw std::invalid_argument("--kernel must be tuned, tuned-exact or plain");
    }
    if (has("seed")) {
        o.seed = std::stoull(str("seed"));
        o.seedGiven = true;
    }
    if (has("de-f")) o.deF = f("de-f");
    if (has("de-cr")) o.deCR = f("de-cr");
    if (has("precision")) {
        std::string p = str("precision");
        if (p == "fp32") o.storage = HPSS_STORAGE_FP32;
        else if (p == "bf16") o.storage = HPSS_STORAGE_BF16;
        else if (p == "fp16") o.storage = HPSS_STORAGE_FP16;
        else throw std::invalid_argument("--precision must be fp32, bf16 or fp16");
    }
    if (has("fp64-traveltime")) o.precisionFlags |= HPSS_PREC_FP64_TRAVELTIME;
    if (has("compensated-sums")) o.precisionFlags |= HPSS_PREC_COMPENSATED;
    if (has("grid-mode")) {
        std::string gm = str("grid-mode");
        if (gm == "reference") o.gridMode = HPSS_GRID_REFERENCE;
        else if (gm == "inclusive") o.gridMode = HPSS_GRID_INCLUSIVE;
        else throw std::invalid_argument("--grid-mode must be reference or inclusive");
    }
    return o;
}

Traveltime *Parser::parseTraveltime() const {
    if (!has("traveltime")) throw std::invalid_argument("Traveltime traveltime not provided.");
    const std::string t = str("traveltime");
    const auto lo = floats("lower-bounds"), hi = floats("upper-bounds");
    if (t == "cmp") return TraveltimeBuilder::buildCommonMidPoint(lo, hi);
    if (t == "zocrs") {
        if (!has("ain") || !has("v0") || !has("bpctg"))
            throw std::invalid_argument("Not all arguments have been provided.");
        return TraveltimeBuilder::buildZeroOffsetCommonReflectionSurface(lo, hi, f("v0"), f("ain"),
                                                                         f("bpctg"));
    }
    if (t == "oct")
        return TraveltimeBuilder::buildOffsetContinuationTrajectory(lo, hi,
                                                                    has("h0") ? f("h0") : 0.f);
    throw std::invalid_argument("Invalid traveltime: " + t);
}

void Parser::printHelp() const {
    std::cout << "Allowed options:" << std::endl;
    for (auto &o : options)
        std::cout << "  --" << std::left << std::setw(20) << o.name << o.help
                  << (o.def.empty() ? "" : " (=" + o.def + ")") << std::endl;
}

void Parser::readGather() const {
    if (!has("apm") || !has("aph") || !has("tau"))
        throw std::invalid_argument("Not all arguments to read the gather have been provided.");
    Gather *g = Gather::getInstance();
    g->setApm(f("apm"));
    g->setAph(f("aph"));
    g->setTau(f("tau"));
    if (has("azimuth")) g->setAzimuthInDegree(f("azimuth"));
    if (has("lowest-midpoint")) g->setLowestAllowedMidpoint(f("lowest-midpoint"));
    if (has("highest-midpoint")) g->setBiggestAllowedMidpoint(f("highest-midpoint"));
    g->readGatherFromFile(getInputFilePath());
}

LinearSearchParser::LinearSearchParser() {
    add("granularity", "Discretization granularities.", true, true);
}
ComputeAlgorithm *LinearSearchParser::parseComputeAlgorithm(ComputeAlgorithmBuilder *b,
                                                            std::shared_ptr<DeviceContext> ctx,
                                                            std::shared_ptr<Traveltime> tt) const {
    return b->buildLinearSearchAlgorithm(tt, ctx, getGpuThreadCount(), ints("granularity"));
}

DifferentialEvolutionParser::DifferentialEvolutionParser() {
    add("generations", "Number of generations to be used in differential evolution.", true);
    add("population-size", "Differential evolution population size.", true);
    add("seed", "Random seed (default: time-based, as the reference).");
    add("de-f", "Mutation factor F (reference: 0.85).");
    add("de-cr", "Crossover rate CR (reference: 0.5).");
}
ComputeAlgorithm *DifferentialEvolutionParser::parseComputeAlgorithm(
    ComputeAlgorithmBuilder *b, std::shared_ptr<DeviceContext> ctx,
    std::shared_ptr<Traveltime> tt) const {
    if (!has("generations") || !has("population-size"))
        throw std::logic_error("Missing parameters for differential evolution.");
    return b->buildDifferentialEvolutionAlgorithm(tt, ctx, getGpuThreadCount(), u("generations"),
                                                  u("population-size"));
}

StretchFreeParser::StretchFreeParser() {
    add("stack-datafiles", "Datafiles to be used for stretch-free stack generation.", true, true);
}
Traveltime *StretchFreeParser::parseTraveltime() const {
    return new StretchFreeTraveltimeWrapper(Parser::parseTraveltime());
}
ComputeAlgorithm *StretchFreeParser::parseComputeAlgorithm(ComputeAlgorithmBuilder *b,
                                                           std::shared_ptr<DeviceContext> ctx,
                                                           std::shared_ptr<Traveltime> tt) const {
    std::vector<std::string> files;
    auto it = values.find("stack-datafiles");
    if (it != values.end()) files = it->second;
    return b->buildStretchFreeAlgorithm(tt, ctx, getGpuThreadCount(), files);
}

// ================================================================ runner
SingleHostRunner::SingleHostRunner(Parser *p) : parser(p) {}

// SingleHostRunner::main (common/src/execution/SingleHostRunner.cpp:108-196),
// with the same exit codes: invalid_argument -> message + help, 0;
// runtime_error -> -ENODEV; anything else -> -1.
int SingleHostRunner::main(int argc, const char *argv[]) {
    try {
        auto start = std::chrono::steady_clock::now();
        int devices = 0;
        parser->parseArguments(argc, argv);
        if (hpss_device_count(&devices) != HPSS_OK || devices == 0)
            throw std::runtime_error("No CUDA devices found on your system. Exiting.");
        Gb300ComputeAlgorithmBuilder builder(parser->engineOptions());
        traveltime.reset(parser->parseTraveltime());
        Dumper dumper(parser->getOutputDirectory(), parser->getFilename(), parser->getParserType(),
                      traveltime->getTraveltimeWord());
        dumper.createDir();
        auto t0 = std::chrono::steady_clock::now();
        parser->readGather();
        auto tRead = std::chrono::steady_clock::now() - t0;
        Gather *gather = Gather::getInstance();
        std::vector<float> m0s;
        for (auto &kv : gather->getCdps()) m0s.push_back(kv.first);
        const unsigned S = gather->getSamplesPerTrace();
        resultSet = std::make_unique<ResultSet>(traveltime->getNumberOfResults(), S);

        const unsigned nDev = std::min<unsigned>((unsigned)devices, std::max<size_t>(m0s.size(), 1));
        std::vector<std::thread> threads;
        std::vector<std::string> errors(nDev);
        std::vector<int> errorKind(nDev, 0);
        std::string algorithmText;
        for (unsigned d = 0; d < nDev; d++) {
            threads.emplace_back([&, d]() {
                try {
                    size_t a = m0s.size() * d / nDev, b = m0s.size() * (d + 1) / nDev;
                    std::vector<float> shard(m0s.begin() + a, m0s.begin() + b);
                    auto ctx = std::make_shared<DeviceContext>(d);
                    std::unique_ptr<ComputeAlgorithm> alg(
                        parser->parseComputeAlgorithm(&builder, ctx, traveltime));
                    alg->setUp();
                    std::vector<float> res;
                    std::vector<std::map<StatisticResult, float>> st;
                    if (!shard.empty()) alg->computeSemblanceAndParametersForMidpoints(shard, res, st);
                    std::lock_guard<std::mutex> lock(resultSetMutex);
                    if (d == 0) algorithmText = alg->toString();
                    const size_t block = (size_t)traveltime->getNumberOfResults() * S;
                    for (size_t i = 0; i < shard.size(); i++) {
                        resultSet->setAllResultsForMidpoint(shard[i], res, i * block);
                        for (auto &kv : st[i])
                            resultSet->setStatisticalResultForMidpoint(shard[i], kv.first, kv.second);
                    }
                } catch (const std::invalid_argument &e) {
                    errors[d] = e.what();
                    errorKind[d] = 1;
                } catch (const std::logic_error &e) {
                    errors[d] = e.what();
                    errorKind[d] = 2;
                } catch (const std::exception &e) {
                    errors[d] = e.what();
                    errorKind[d] = 3;
                }
            });
        }
        for (auto &t : threads) t.join();
        for (unsigned d = 0; d < nDev; d++) {
            if (errorKind[d] == 1) throw std::invalid_argument(errors[d]);
            if (errorKind[d] == 2) throw std::logic_error(errors[d]);
            if (errorKind[d] == 3) throw std::runtime_error(errors[d]);
        }
        dumper.dumpGatherParameters(parser->getInputFilePath());
        dumper.dumpTraveltime(traveltime.get());
        {
            std::ofstream o(dumper.getOutputDirectoryPath() + "algorithm.txt");
            o << "==== Compute Algorithm Summary ====" << std::endl << algorithmText << std::endl;
        }
        for (unsigned i = 0; i < traveltime->getNumberOfResults(); i++)
            dumper.dumpResult(traveltime->getDescriptionForResult(i), resultSet->getArrayForResult(i));
        if (!m0s.empty()) {
            for (int i = 0; i < (int)StatisticResult::CNT; i++) {
                auto sr = static_cast<StatisticResult>(i);
                dumper.dumpStatisticalResult(statisticName(sr), resultSet->get(sr));
                LOGI("Average of " << statisticName(sr) << " is "
                                   << resultSet->get(sr).getAverageOfAllMidpoints());
            }
        }
        auto total = std::chrono::steady_clock::now() - start;
        LOGI("Read gather duration is " << std::chrono::duration<double>(tRead).count() << " s");
        LOGI("Results written to " << dumper.getOutputDirectoryPath());
        LOGI("It took " << std::chrono::duration<double>(total).count() << " s to compute.");
        return 0;
    } catch (const std::invalid_argument &e) {
        std::cout << e.what() << std::endl;
        parser->printHelp();
        return 0;
    } catch (const std::runtime_error &e) {
        std::cout << e.what() << std::endl;
        return -ENODEV;
    } catch (const std::exception &e) {
        std::cout << e.what() << std::endl;
        return -1;
    }
}

}  // namespace hpsshost
