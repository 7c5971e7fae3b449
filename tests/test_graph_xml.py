"""Graph files (Graph::Serialize / Deserialize, ptask/graph.h:1545-1561): the FDTD graph's structure in
the reference's XML layout (ptask/XMLWriter.cpp:124-588, XMLReader.cpp:383-1083).  CPU only: the
graphs are built and written without a device (ptk_fdtd_graph_export) and read back into a new graph
(ptk_graph_xml_roundtrip).  Running a loaded graph is tested in test_graph_gpu.py."""
import re
import xml.etree.ElementTree as ET

import pytest

import ptask_gb300 as P
from ptask_gb300 import graph as G

SECTIONS = ["DatablockTemplates", "CompiledKernels", "Tasks", "Channels", "Actions"]
REF_ACTIONS = {"SetComputeGeometry", "SetBlockAndGridSize", "SetPredicationType", "BindControlPropagationPort",
               "BindControlPropagationChannel", "BindIterationScope", "BindDescriptorPort", "BindControlPort"}


def export(tmp_path, mode, steps=0, shape=(8, 6, 5)):
    path = tmp_path / f"{mode}.xml"
    G.export_graph(P.reference_params(*shape), path, mode, steps)
    return path


def actions(root):
    return [a.findtext("ActionName") for a in root.find("Actions").findall("Action")]


def test_unrolled_graph_layout_matches_reference_writer(tmp_path):
    root = ET.parse(export(tmp_path, "unrolled", 2)).getroot()
    assert root.tag == "Graph" and [c.tag for c in root] == SECTIONS
    for sec, item in zip(SECTIONS, ["DatablockTemplate", "CompiledKernel", "Task", "Channel", "Action"]):
        assert int(root.find(sec).findtext("Count")) == len(root.find(sec).findall(item))
    t = root.find("DatablockTemplates").findall("DatablockTemplate")
    assert [c.tag for c in t[0]] == ["Name", "Stride", "ParamType", "ElementsX", "ElementsY", "ElementsZ",
                                     "IsRecordStream", "IsByteAddressable"]
    dims = {x.findtext("Name"): (int(x.findtext("ElementsX")), int(x.findtext("ElementsY")),
                                 int(x.findtext("ElementsZ"))) for x in t}
    assert dims["HxSize"] == (9, 6, 5) and dims["EzSize"] == (9, 7, 5)          # graphfdtd.cpp:70-85
    kernels = sorted(k.findtext("Operation") for k in root.find("CompiledKernels").findall("CompiledKernel"))
    assert kernels == sorted(f + "Computation" for f in ("Hx", "Hy", "Hz", "Ex", "Ey", "Ez"))
    tasks = root.find("Tasks").findall("Task")
    assert len(tasks) == 12
    for task in tasks:
        assert [c.tag for c in task] == ["Name", "KernelID", "AcceleratorClass", "InputPorts", "OutputPorts"]
        ins = task.find("InputPorts").findall("Port")
        assert len(ins) == 4 and len(task.find("OutputPorts").findall("Port")) == 1
        assert [c.tag for c in ins[0]] == ["UniqueID", "OriginalIndex", "Type", "DatablockTemplate",
                                           "VariableBinding", "ParameterIndex", "InOutIndex"]
        assert ins[3].findtext("VariableBinding") == "Config" and ins[3].findtext("Type") == "2"   # STICKY_PORT
    ch = root.find("Channels").findall("Channel")
    types = [int(c.findtext("Type")) for c in ch]
    # per step: 6 Config inputs + 6 H->E + 12 field inputs (graph inputs in step 1); 6 outputs at the end
    assert types.count(0) == 12 + 12 and types.count(2) == 12 + 12 and types.count(1) == 6
    assert all(c.findtext("SourcePort") == "-1" for c in ch if c.findtext("Type") == "0")
    acts = actions(root)
    assert acts.count("SetComputeGeometry") == 12


def test_cyclic_graph_records_iteration_state(tmp_path):
    root = ET.parse(export(tmp_path, "fused")).getroot()
    acts = actions(root)
    assert acts.count("SetPredicationType") == 12          # 6 back channels + 6 outputs
    assert acts.count("BindControlPropagationPort") == 6
    assert acts.count("SetMetaFunction") == 1 and acts.count("SetSwitchChannel") == 6
    meta = [a for a in root.find("Actions").findall("Action") if a.findtext("ActionName") == "SetMetaFunction"]
    assert meta[0].findtext("MetaFunction") == "3"          # MF_GENERAL_ITERATOR


@pytest.mark.parametrize("mode,steps", [("unrolled", 3), ("fused", 0)])
def test_roundtrip_is_exact(tmp_path, mode, steps):
    a = export(tmp_path, mode, steps)
    b = tmp_path / "again.xml"
    G.xml_roundtrip(a, b)
    assert b.read_text() == a.read_text()


def reference_style(text: str) -> str:
    """The same graph laid out the way the reference's writer leaves it: only the reference's
    action kinds, no indentation, CRLF line ends, and channel names unlike this runtime's builder
    (the reference's driver uses its own, graphfdtd.cpp:617-700)."""
    root = ET.fromstring(text)
    acts = root.find("Actions")
    for a in list(acts.findall("Action")):
        if a.findtext("ActionName") not in REF_ACTIONS:
            acts.remove(a)
    acts.find("Count").text = str(len(acts.findall("Action")))
    for n, c in enumerate(root.find("Channels").findall("Channel")):
        c.find("Name").text = f"Channel_{n}_" + c.findtext("Name")
    body = ET.tostring(root, encoding="unicode")
    body = re.sub(r">\s+<", "><", body).replace("><", ">\r\n<")
    return '<?xml version="1.0" encoding="utf-8"?>\r\n<!-- written by another tool -->\r\n' + body


def test_reference_layout_without_extensions_loads(tmp_path):
    src = export(tmp_path, "unrolled", 2)
    ref = tmp_path / "ref_style.xml"
    ref.write_text(reference_style(src.read_text()))
    out = tmp_path / "out.xml"
    G.xml_roundtrip(ref, out)
    root = ET.parse(out).getroot()
    assert len(root.find("Tasks").findall("Task")) == 12 and len(root.find("Channels").findall("Channel")) == 54
    assert set(actions(root)) == {"SetComputeGeometry"}


@pytest.mark.parametrize("damage", ["truncate", "count", "action", "port", "root"])
def test_malformed_files_are_rejected(tmp_path, damage):
    text = export(tmp_path, "fused").read_text()
    if damage == "truncate":
        text = text[: len(text) // 2]
    elif damage == "count":
        text = text.replace("<Count>2</Count>", "<Count>3</Count>", 1)
    elif damage == "action":
        text = text.replace("<ActionName>SetNoDraw</ActionName>", "<ActionName>Frobnicate</ActionName>", 1)
    elif damage == "port":
        text = re.sub(r"<DestinationPort>\d+</DestinationPort>", "<DestinationPort>99999</DestinationPort>", text,
                      count=1)
    else:
        text = text.replace("<Graph>", "<Grape>").replace("</Graph>", "</Grape>")
    bad = tmp_path / "bad.xml"
    bad.write_text(text)
    with pytest.raises(P.PtkError):
        G.xml_roundtrip(bad, tmp_path / "out.xml")


def test_missing_file_is_an_error(tmp_path):
    with pytest.raises(P.PtkError):
        G.xml_roundtrip(tmp_path / "absent.xml", tmp_path / "out.xml")
