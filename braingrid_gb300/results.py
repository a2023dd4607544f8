"""The reference's simulation result file: XmlGrowthRecorder::saveSimData
(Recorders/XmlGrowthRecorder.cpp:104-153) for ConnGrowth networks, XmlRecorder::saveSimData
(Recorders/XmlRecorder.cpp:111-160) for the others, written byte for byte.

Each matrix is written as CompleteMatrix::toXML / VectorMatrix::toXML do (Matrix/
CompleteMatrix.cpp:225-249, Matrix/VectorMatrix.cpp:173-190): an opening tag, three spaces, the
values each followed by one space (a complete matrix ends every row with a newline), a newline,
the closing tag.  Values are BGFLOAT written by an ostream at its default precision, i.e. C's %g
with six significant digits of the float widened to double.
"""
import numpy as np

_HEADER = ('<?xml version="1.0" standalone="no"?>\n'
           '<!-- State output file for the DCT growth modeling-->\n<SimState>\n')


def _g(v):
    return "%g" % float(np.float32(v))


def vector_xml(name, values):
    values = np.asarray(values).ravel()
    return ('<Matrix name="%s" type="complete" rows="1" columns="%d" multiplier="1.0">\n   %s\n'
            '</Matrix>' % (name, values.size, "".join(_g(v) + " " for v in values)))


def complete_xml(name, values):
    values = np.asarray(values)
    rows = "".join("".join(_g(v) + " " for v in row) + "\n" for row in values)
    return ('<Matrix name="%s" type="complete" rows="%d" columns="%d" multiplier="1.0">\n   %s\n'
            '</Matrix>' % (name, values.shape[0], values.shape[1], rows))


def _scalar(name, text):
    return ('   <Matrix name="%s" type="complete" rows="1" columns="1" multiplier="1.0">\n'
            '   %s\n</Matrix>\n' % (name, text))


def state_xml(growth, n_neurons, epochs, epoch_duration, delta_t, sim_step, histories, xloc,
              yloc, ntype, starter, vthresh):
    """The result file's text.  growth: ConnGrowth's recorder (radii and rates histories first);
    histories: (burstiness, spikes, rates, radii) as bg3_download_histories returns them (the
    rates and radii histories (epochs + 1) x N, row 0 the start values); sim_step: the
    simulation step at the end (g_simulationStep); starter: bool per neuron."""
    burst, spikes, rates, radii = histories
    N = n_neurons
    out = [_HEADER]
    if growth:
        out.append("   " + complete_xml("radiiHistory",
                                        np.asarray(radii)[:(epochs + 1) * N].reshape(-1, N)) + "\n")
        out.append("   " + complete_xml("ratesHistory",
                                        np.asarray(rates)[:(epochs + 1) * N].reshape(-1, N)) + "\n")
    out.append("   " + vector_xml("burstinessHist", burst) + "\n")
    out.append("   " + vector_xml("spikesHistory", spikes) + "\n")
    out.append("   " + vector_xml("xloc", xloc) + "\n")
    out.append("   " + vector_xml("yloc", yloc) + "\n")
    out.append("   " + vector_xml("neuronTypes", ntype) + "\n")
    st = np.nonzero(np.asarray(starter))[0]
    if st.size:
        out.append("   " + vector_xml("starterNeurons", st) + "\n")
    out.append("   " + vector_xml("neuronThresh", vthresh) + "\n")
    out.append(_scalar("Tsim", _g(epoch_duration)))
    # g_simulationStep * deltaT: the step count converted to float, times the float deltaT
    out.append(_scalar("simulationEndTime", _g(np.float32(sim_step) * np.float32(delta_t))))
    out.append("</SimState>\n")
    return "".join(out)
