"""Task files for the driver tests, in the form the reference's scripted tests write them
(test/scripted/test_*.sh): manual or exponential frequencies, exponential cutoffs, one
lattice, one model and a correlation measurement."""

REFERENCE_FREQUENCIES = (0.31812, 0.36329, 0.41812, 0.46329, 0.51334, 0.56880, 0.63024, 0.69833, 0.77378,
                         0.85737, 0.95, 1.0, 3.0, 10.0)


def manual_frequencies(values=REFERENCE_FREQUENCIES):
    return '<frequency discretization="manual">' + "".join(f"<value>{v}</value>" for v in values) + "</frequency>"


def exponential_cutoffs(cmax, cmin, step):
    return f'<cutoff discretization="exponential"><max>{cmax}</max><min>{cmin}</min><step>{step}</step></cutoff>'


def task_xml(lattice="square", rng=2, model="square-heisenberg", symmetry="SU2", params="<j>1.0</j>",
             freq=manual_frequencies((0.31812, 0.36329, 0.41812, 1.0, 3.0, 10.0)),
             cutoff=exponential_cutoffs(10, 0.3, 0.9),
             measurements='<measurements><measurement name="correlation" /></measurements>', extra=""):
    return f"""<?xml version="1.0" encoding="utf-8"?>
<task>
    <parameters>
        {freq}
        {cutoff}
        <lattice name="{lattice}" range="{rng}"/>
        <model name="{model}" symmetry="{symmetry}">{params}</model>
    </parameters>
    {measurements}
    {extra}
</task>
"""


def write(tmp_path, name="t.xml", **kw):
    p = tmp_path / name
    p.write_text(task_xml(**kw))
    return str(p)
