// Stand-in for the reference's VisIt writer: plotting is not built (no HDF5), so the flow
// models' registerPlotQuantities (compiled only with HAVE_HDF5) never refers to it.
#ifndef EXTENDED_VISIT_DATA_WRITER_HPP
#define EXTENDED_VISIT_DATA_WRITER_HPP

class ExtendedVisItDataWriter;

#endif
