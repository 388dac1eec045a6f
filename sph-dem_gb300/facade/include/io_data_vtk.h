/*
 * Restart and output files of a case (the reference's Cio_data_vtk,
 * io_data_vtk.h): VTK XML UnstructuredGrid pieces written and read without
 * the VTK library.
 *
 *   <base>Restart%07d_<rank>.vtu + <base>Restart%07d.pvtu   restart
 *   <base>%07d_<rank>.vtu + <base>%07d.pvtu                 output
 *
 * The point arrays are the reference's, in its order (io_data_vtk.cpp:231-411):
 * dens, h, eBForce, eViscF, eViscB, eFF, u, mass, colour, iam, tag, v, vhat,
 * vort, norm1, norm2 (, norm3), binary, base64, with the
 * vtkZLibDataCompressor block header when zlib is available (else raw
 * base64 with the UInt32 byte-count header).  Positions are the points:
 * Float32 as VTK writes them for the reference, or Float64 with
 * setExactPoints(true).  The reader accepts either, compressed or not, and
 * ignores arrays it does not use (readRestart, io_data_vtk.cpp:20-114).
 */
#ifndef SPHDEM_FACADE_IO_DATA_VTK_H
#define SPHDEM_FACADE_IO_DATA_VTK_H

#include <string>
#include <vector>

#include "globalVars.h"
#include "particle.h"

class Cio_data_vtk {
   public:
    Cio_data_vtk() {}
    Cio_data_vtk(const std::string &fn, CglobalVars *) : filename(fn) {}
    void setFilename(const std::string &fn, CglobalVars *) { filename = fn; }
    std::string getFilename() const { return filename; }
    /* Float64 points (a restart that continues a run exactly) */
    void setExactPoints(bool e) { exactPoints = e; }

    /* the reference's entry points (rank = globals->mpiRank) */
    void readRestart(int timestep, particleContainer *outPs, CglobalVars *globals);
    void writeRestart(int timestep, particleContainer &ps, CglobalVars *globals);
    /* the output pieces <base>%07d in the restart layout above; the
     * reference's visualisation output (io_data_vtk.cpp:413-720: Float32
     * press, porosity, shepSum, fdrag, force parts, ...) is not written */
    void writeOutput(int timestep, particleContainer &ps, CglobalVars *globals);

    /* <filename>Globals<rank>.dat (CioGlobals, ioGlobals.cpp:4-139): one
     * row per output step.  readGlobals reads the rows up to the one of
     * outStep into g (none for outStep 0); writeGlobals keeps the rows up
     * to outStep - 1 and writes g as the row of outStep, creating the file
     * with the reference's header line.  Numbers are written to full
     * precision. */
    void readGlobals(int outStep, CglobalVars *g);
    void writeGlobals(int outStep, CglobalVars *g);
    /* <filename>Domain<rank>.dat (CioDomain, ioDomain.cpp:3-40): rank,
     * procDomain[2 NDIM], procNeighbrs[3^NDIM]; readDomain returns false
     * when the file cannot be read */
    bool readDomain(int outStep, CglobalVars *g);
    void writeDomain(int outStep, CglobalVars *g);

    /* one piece by path; readPiece returns false (with a message on stderr)
     * when the file cannot be read */
    static bool readPiece(const std::string &path, particleContainer &ps);
    static bool writePiece(const std::string &path, const particleContainer &ps, bool float64Points);
    static void writeIndex(const std::string &path, const std::vector<std::string> &pieces, bool float64Points);

    std::string filename;

   private:
    bool exactPoints = false;
};

#endif
